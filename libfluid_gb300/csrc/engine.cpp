// Host-side engine (see engine.h).
#include "engine.h"

#include "arena_policy.h"

#include <algorithm>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>

namespace sph {

namespace {
constexpr float PI_F = 3.141592654f;   // fluiddefines.h:16 (CUDART_PI_F)
const char* kPassNames[Engine::kPasses] = {"hash", "scan", "sort", "density", "normals", "force_integrate",
                                           "xsph", "substep"};
}  // namespace

bool derive_params(const SceneConfig& c, DevParams& d, std::string* err) {
    std::memset(&d, 0, sizeof(d));
    float h;
    if (c.box_mode == 0) {
        if (c.res == 0) { if (err) *err = "res must be positive"; return false; }
        d.gx = d.gy = d.gz = c.res;
        d.inv_cell = float(c.res);                      // grid_from_point multiplies by m_res (fluidutil.cu:17)
        d.box_cx = d.box_cy = d.box_cz = 0.5f;          // unit cube SDF (fluidutil.cu:87)
        d.box_bx = d.box_by = d.box_bz = 0.5f;
        h = 1.0f / float(c.res);                        // fluidparams.cu:62
    } else {
        if (!(c.h > 0.f) || !(c.lx > 0.f) || !(c.ly > 0.f) || !(c.lz > 0.f)) {
            if (err) *err = "box extents and h must be positive";
            return false;
        }
        // cells per axis: ceil(l/h), tolerant to the float rounding of h
        auto cells = [&](float l) -> uint32_t {
            const double v = std::ceil(double(l) / double(c.h) - 1e-3);
            return v < 1.0 ? 1u : (uint32_t)v;
        };
        d.gx = cells(c.lx); d.gy = cells(c.ly); d.gz = cells(c.lz);
        d.inv_cell = 1.0f / c.h;
        d.box_cx = d.box_bx = 0.5f * c.lx;
        d.box_cy = d.box_by = 0.5f * c.ly;
        d.box_cz = d.box_bz = 0.5f * c.lz;
        h = c.h;
    }
    const uint64_t cells = (uint64_t)d.gx * d.gy * d.gz;
    if (cells >= (1ull << 31)) { if (err) *err = "grid too large"; return false; }
    d.gxy = d.gx * d.gy;
    d.ncells = (uint32_t)cells;
    // fluidparams.cu:63-86
    d.h = h;
    d.halfh = 0.5f * h;
    d.h2 = h * h;
    const float h3 = h * h * h;
    d.h4 = h * h * h * h;
    const float h5 = h3 * d.h2;
    d.h6 = h3 * h3;
    d.h8 = h5 * h3;
    d.h9 = d.h6 * h3;
    d.invh9 = 1.0f / (d.h6 * h3);
    d.poly6 = 315.0f / (64.0f * PI_F * powf(h, 9.0f));
    d.grad_poly6 = -945.0f / (32.0f * PI_F * powf(h, 9.0f));
    d.grad_spiky = -45.0f / (PI_F * powf(h, 6.0f));
    d.cohesion = 32.0f / (PI_F * powf(h, 9.0f));
    d.visc_eps = (float)(0.01 * (double)d.h2);
    // fluid parameters (fluidparams.cu:99-213)
    d.rest_density = c.rest_density;
    d.inv_rest_density = (c.rest_density == 0.0f) ? 1.0f : 1.0f / c.rest_density;
    d.gas_constant = c.gas_constant;
    d.gamma = c.gamma;
    const float inv_gamma = (c.gamma == 0.0f) ? 1.0f : 1.0f / c.gamma;
    d.eos_k = c.gas_constant * c.rest_density * inv_gamma;
    d.mass = c.mass;
    d.two_mass = 2.0f * c.mass;
    d.particle_size = c.particle_size;
    d.inv_particle_size = 1.0f / c.particle_size;
    d.dt = c.dt;
    d.dtdt = c.dt * c.dt;
    d.xsph = c.xsph;
    d.surface_tension = c.surface_tension;
    d.viscosity = c.viscosity;
    d.adhesion = c.adhesion;
    d.vdamp = c.vdamp;
    d.vel_limit = c.vel_limit;
    d.acc_limit = c.acc_limit;
    d.vel_limit2 = c.vel_limit * c.vel_limit;
    d.acc_limit2 = c.acc_limit * c.acc_limit;
    d.grav_x = c.gravity[0]; d.grav_y = c.gravity[1]; d.grav_z = c.gravity[2];
    d.eps = FLT_MIN;
    d.flags = (c.surface_tension != 0.0f) ? 1u : 0u;
    if (c.boundary != 0 && c.boundary != 1) { if (err) *err = "boundary must be 0 (box) or 1 (sphere)"; return false; }
    if (c.boundary == 1) d.flags |= SPH_FLAG_SPHERE;
    d.sphere_r = std::fmin(d.box_bx, std::fmin(d.box_by, d.box_bz));
    const float skin = (c.skin > 0.0f) ? c.skin : SPH_SKIN_DEFAULT;
    const float rs = (1.0f + skin) * h;
    d.skin2 = rs * rs;
    d.inv_h2 = 1.0f / d.h2;
    d.xsph_disp_limit2 = 0.25f * skin * skin * 0.98f;
    return true;
}

uint64_t Engine::bytes_per_particle() { return 10 * 16 + 5 * 4 + SPH_MASK_ROWS * 4; }
uint64_t Engine::bytes_per_cell() { return 2 * 4 + 1; }
const char* Engine::pass_name(int i) { return (i >= 0 && i < kPasses) ? kPassNames[i] : "?"; }

Engine::Engine(int device) {
    if (device < 0) cudaGetDevice(&device_);
    else device_ = device;
    cudaSetDevice(device_);
    cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&copy_ev_, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&suffix_ev_, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&pack_ev_, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&vel_ev_, cudaEventDisableTiming);
    cudaMallocHost((void**)&h_status_, sizeof(uint32_t));
    cudaMalloc((void**)&status_, 2 * sizeof(uint32_t));
    cudaMemsetAsync(status_, 0, 2 * sizeof(uint32_t), stream_);
    gate_ = status_ + 1;
    cudaMalloc((void**)&scal_, 8 * sizeof(uint32_t));
    cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device_);
    for (auto& e : ev_) cudaEventCreate(&e);
    init_kernel_attributes();   // a performance hint only: launches work without it
}

Engine::~Engine() {
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    if (copy_stream_) cudaStreamSynchronize(copy_stream_);
    free_all();
    for (cudaGraphExec_t e : {exec_pre_, exec_suf_, exec_full_})
        if (e) cudaGraphExecDestroy(e);
    for (cudaGraph_t g : {graph_pre_, graph_suf_, graph_full_})
        if (g) cudaGraphDestroy(g);
    for (auto& e : ev_) if (e) cudaEventDestroy(e);
    for (auto& e : timers_) if (e) cudaEventDestroy(e);
    if (status_) cudaFree(status_);
    if (scal_) cudaFree(scal_);
    if (h_status_) cudaFreeHost(h_status_);
    if (h_params_) cudaFreeHost(h_params_);
    if (copy_ev_) cudaEventDestroy(copy_ev_);
    if (suffix_ev_) cudaEventDestroy(suffix_ev_);
    if (pack_ev_) cudaEventDestroy(pack_ev_);
    if (vel_ev_) cudaEventDestroy(vel_ev_);
    if (copy_stream_) cudaStreamDestroy(copy_stream_);
    if (stream_) cudaStreamDestroy(stream_);
}

int Engine::fail(int code, const std::string& msg) {
    err_ = msg;
    return code;
}
int Engine::cuda_fail(cudaError_t e, const char* what) {
    err_ = std::string(what) + ": " + cudaGetErrorString(e);
    return ENG_ECUDA;
}
#define ENG_CK(expr, what)                       \
    do {                                         \
        cudaError_t e__ = (expr);                \
        if (e__ != cudaSuccess) return cuda_fail(e__, what); \
    } while (0)

void Engine::free_all() {
    float4** f4[] = {&P0_, &P1_, &V0_, &V1_, &V2_, &A0_, &A1_, &S_, &N_, &Vc_, &dbg_forces_};
    for (auto p : f4) { if (*p) cudaFree(*p); *p = nullptr; }
    uint32_t** u[] = {&key_, &slot_, &tmp_, &perm_, &count_, &start_, &scan_sums_, &dbg_nbr_, &mask_,
                      &okey_, &pend_};
    for (auto p : u) { if (*p) cudaFree(*p); *p = nullptr; }
    if (stage_) cudaFree(stage_);
    stage_ = nullptr;
    stage_bytes_ = 0;
    if (d_params_) cudaFree(d_params_);
    if (d_scenes_) cudaFree(d_scenes_);
    if (d_tiles_) cudaFree(d_tiles_);
    if (d_tile_first_) cudaFree(d_tile_first_);
    d_params_ = nullptr; d_scenes_ = nullptr; d_tiles_ = nullptr; d_tile_first_ = nullptr;
    pcap_ = ccap_ = 0;
    scene_cap_ = tile_cap_ = tile_first_cap_ = pend_cap_ = 0;
    dev_bytes_ = 0;
}

// Grow the particle and cell arenas, preserving live particle state.
int Engine::ensure_capacity(uint64_t parts, uint64_t cells) {
    cudaSetDevice(device_);
    // sizes under the memory budget (arena_policy.h)
    const ArenaPlan plan = plan_arena(parts, cells, pcap_, ccap_, byte_limit_, bytes_per_particle());
    if (plan.status == kArenaOverBudget) return fail(ENG_ENOMEM, "arena would exceed the memory budget");
    if (plan.status == kArenaAtBudget) return fail(ENG_ENOMEM, "arena at its memory budget");
    if (plan.parts > pcap_) {
        const uint64_t np = plan.parts;
        if (np >= (1ull << 31)) return fail(ENG_ENOMEM, "particle capacity exceeds 2^31");
        // state between substeps: P0, V0, A0, S, and for scenes with a
        // pending XSPH update their post-integration velocities V2 and cells
        float4** state[] = {&P0_, &V0_, &A0_, &S_, &V2_};
        float4** scratch[] = {&P1_, &V1_, &A1_, &N_, &Vc_};
        for (auto p : state) {
            float4* q = nullptr;
            cudaError_t e = cudaMalloc((void**)&q, np * sizeof(float4));
            if (e != cudaSuccess) return fail(ENG_ENOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
            if (*p) {
                ENG_CK(cudaMemcpyAsync(q, *p, pcap_ * sizeof(float4), cudaMemcpyDeviceToDevice, stream_), "grow copy");
                ENG_CK(cudaStreamSynchronize(stream_), "grow sync");
                cudaFree(*p);
            }
            *p = q;
        }
        {
            uint32_t* q = nullptr;
            cudaError_t e = cudaMalloc((void**)&q, np * sizeof(uint32_t));
            if (e != cudaSuccess) return fail(ENG_ENOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
            if (okey_) {
                ENG_CK(cudaMemcpyAsync(q, okey_, pcap_ * sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream_), "grow copy");
                ENG_CK(cudaStreamSynchronize(stream_), "grow sync");
                cudaFree(okey_);
            }
            okey_ = q;
        }
        prefix_valid_ = false;
        for (auto p : scratch) {
            if (*p) cudaFree(*p);
            *p = nullptr;
            cudaError_t e = cudaMalloc((void**)p, np * sizeof(float4));
            if (e != cudaSuccess) return fail(ENG_ENOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
        }
        uint32_t** u[] = {&key_, &slot_, &tmp_, &perm_};
        for (auto p : u) {
            if (*p) cudaFree(*p);
            *p = nullptr;
            cudaError_t e = cudaMalloc((void**)p, np * sizeof(uint32_t));
            if (e != cudaSuccess) return fail(ENG_ENOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
        }
        if (mask_) cudaFree(mask_);
        mask_ = nullptr;
        {
            cudaError_t e = cudaMalloc((void**)&mask_, (size_t)SPH_MASK_ROWS * np * sizeof(uint32_t));
            if (e != cudaSuccess) return fail(ENG_ENOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
        }
        if (dbg_nbr_) { cudaFree(dbg_nbr_); dbg_nbr_ = nullptr; }
        if (dbg_forces_) { cudaFree(dbg_forces_); dbg_forces_ = nullptr; }
        if (debug_) {
            ENG_CK(cudaMalloc((void**)&dbg_nbr_, np * sizeof(uint32_t)), "debug alloc");
            ENG_CK(cudaMalloc((void**)&dbg_forces_, np * 4 * sizeof(float4)), "debug alloc");
        }
        pcap_ = np;
        graph_dirty_ = true;
    }
    if (plan.cells > ccap_) {
        const uint64_t nc = plan.cells;
        if (count_) cudaFree(count_);
        if (start_) cudaFree(start_);
        if (scan_sums_) cudaFree(scan_sums_);
        count_ = start_ = scan_sums_ = nullptr;
        cudaError_t e1 = cudaMalloc((void**)&count_, nc * sizeof(uint32_t));
        cudaError_t e2 = cudaMalloc((void**)&start_, (nc + 1) * sizeof(uint32_t));
        // the scan's tile counter and look-back descriptors (64-bit words)
        cudaError_t e3 = cudaMalloc((void**)&scan_sums_, (nc / 4096 + 3) * sizeof(unsigned long long));
        if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
            return fail(ENG_ENOMEM, "device allocation of cell arrays failed");
        ccap_ = nc;
        graph_dirty_ = true;
        prefix_valid_ = false;
    }
    dev_bytes_ = pcap_ * bytes_per_particle() + ccap_ * 8;
    return ENG_OK;
}

uint32_t Engine::alloc_slots(uint32_t n) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= n) {
            const uint32_t base = it->first;
            const uint32_t rest = it->second - n;
            free_.erase(it);
            if (rest) free_[base + n] = rest;
            return base;
        }
    }
    const uint32_t base = (uint32_t)slots_end_;
    slots_end_ += n;
    return base;
}

void Engine::free_slots(uint32_t base, uint32_t n) {
    if (n == 0) return;
    if ((uint64_t)base + n == slots_end_) {
        slots_end_ = base;
        // merge a trailing free range
        while (!free_.empty()) {
            auto last = std::prev(free_.end());
            if ((uint64_t)last->first + last->second == slots_end_) {
                slots_end_ = last->first;
                free_.erase(last);
            } else break;
        }
        return;
    }
    auto it = free_.emplace(base, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
    if (it != free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
    }
}

int Engine::staging(size_t bytes, float** out) {
    if (bytes > stage_bytes_) {
        if (stage_) { cudaStreamSynchronize(stream_); cudaStreamSynchronize(copy_stream_); cudaFree(stage_); }
        stage_ = nullptr;
        stage_bytes_ = 0;
        ENG_CK(cudaMalloc((void**)&stage_, bytes), "staging alloc");
        stage_bytes_ = bytes;
    }
    *out = stage_;
    return ENG_OK;
}

uint64_t Engine::total_particles() const {
    uint64_t t = 0;
    for (const auto& s : scenes_) t += s.n;
    return t;
}

const Scene* Engine::scene(int id) const {
    for (const auto& s : scenes_) if (s.id == id) return &s;
    return nullptr;
}

int Engine::set_exec(const ExecConfig& e) {
    if (e.tile != 64 && e.tile != 128 && e.tile != 256) return fail(ENG_EINVAL, "tile must be 64, 128 or 256");
    if (!(e.skin > 0.0f && e.skin <= 1.0f)) return fail(ENG_EINVAL, "skin must be in (0, 1]");
    if (e.persistent > 64) return fail(ENG_EINVAL, "persistent blocks per SM must be <= 64");
    if (e.variant & ~SPH_VARIANT_MASK) return fail(ENG_EINVAL, "unknown kernel variant bits");
    if (const int rc = settle()) return rc;
    if (e.tile != exec_.tile) layout_dirty_ = true;
    graph_dirty_ = true;
    exec_ = e;
    for (auto& s : scenes_) {
        s.cfg.skin = e.skin;
        derive_params(s.cfg, s.dp, nullptr);
    }
    params_dirty_ = true;
    return ENG_OK;
}

int Engine::add_scene(const SceneConfig& cfg_in, uint32_t n, int* id_out) {
    if (const int rc = settle()) return rc;
    Scene s;
    std::string e;
    SceneConfig cfg = cfg_in;
    cfg.skin = exec_.skin;
    if (!derive_params(cfg, s.dp, &e)) return fail(ENG_EINVAL, e);
    if (n == 0) return fail(ENG_EINVAL, "a scene needs at least one particle");
    s.cfg = cfg;
    s.n = n;
    s.id = next_id_++;
    s.part_base = alloc_slots(n);
    uint64_t cells = 0;
    for (const auto& t : scenes_) cells += t.dp.ncells + 1ull;
    cells += s.dp.ncells + 1ull;
    int rc = ensure_capacity(slots_end_, cells);
    if (rc) { free_slots(s.part_base, n); return rc; }
    scenes_.push_back(s);
    layout_dirty_ = params_dirty_ = true;
    prefix_valid_ = false;
    if (id_out) *id_out = s.id;
    return ENG_OK;
}

int Engine::remove_scene(int id) {
    if (const int rc = settle()) return rc;
    for (size_t k = 0; k < scenes_.size(); ++k) {
        if (scenes_[k].id == id) {
            free_slots(scenes_[k].part_base, scenes_[k].n);
            scenes_.erase(scenes_.begin() + k);
            layout_dirty_ = params_dirty_ = true;
            prefix_valid_ = false;
            return ENG_OK;
        }
    }
    return fail(ENG_EINVAL, "unknown scene id");
}

int Engine::set_config(int id, const SceneConfig& cfg_in) {
    SceneConfig cfg = cfg_in;
    cfg.skin = exec_.skin;
    for (auto& s : scenes_) {
        if (s.id != id) continue;
        DevParams dp;
        std::string e;
        if (!derive_params(cfg, dp, &e)) return fail(ENG_EINVAL, e);
        if (std::memcmp(&dp, &s.dp, sizeof(DevParams)) == 0 && dp.ncells == s.dp.ncells) {
            s.cfg = cfg;
            return ENG_OK;
        }
        // a pending XSPH update belongs to the substep that ran with the old
        // parameters: apply it before they change
        if (const int rc = settle()) return rc;
        if (s.pending) { int rc = materialize(s); if (rc) return rc; }
        prefix_valid_ = false;
        if (dp.ncells != s.dp.ncells || dp.flags != s.dp.flags) layout_dirty_ = true;
        s.cfg = cfg;
        if (std::memcmp(&dp, &s.dp, sizeof(DevParams)) != 0) params_dirty_ = true;
        s.dp = dp;
        if (layout_dirty_) {
            uint64_t cells = 0;
            for (const auto& t : scenes_) cells += t.dp.ncells + 1ull;
            int rc = ensure_capacity(slots_end_, cells);
            if (rc) return rc;
        }
        return ENG_OK;
    }
    return fail(ENG_EINVAL, "unknown scene id");
}

int Engine::rebuild_layout() {
    cudaSetDevice(device_);
    const size_t ns = scenes_.size();
    h_scenes_.resize(ns);
    h_tile_first_.resize(ns);
    cell_base_.resize(ns);
    uint64_t cb = 0;
    ntiles_ = 0;
    any_tension_ = false;
    std::vector<uint32_t> h_pend(ns);
    for (size_t k = 0; k < ns; ++k) {
        Scene& s = scenes_[k];
        cell_base_[k] = (uint32_t)cb;
        h_scenes_[k] = DevScene{s.part_base, s.n, (uint32_t)cb, s.dp.ncells};
        cb += s.dp.ncells + 1ull;
        const uint32_t tile = exec_.tile;
        s.table_index = (uint32_t)k;
        s.tile_first = ntiles_;
        s.tile_count = (s.n + tile - 1u) / tile;
        h_tile_first_[k] = s.tile_first;
        ntiles_ += s.tile_count;
        any_tension_ = any_tension_ || (s.dp.flags & 1u);
        h_pend[k] = s.pending ? 1u : 0u;
    }
    // cells are indexed with u32 (keys, starts, and the scan's tile
    // arithmetic, which rounds up to whole 4096-cell tiles)
    if (cb > 0xFFFFFFFFull - 2ull * kScanTileCells)
        return fail(ENG_ENOMEM, "the live scenes need more than 2^32 - 8192 grid cells");
    total_cells_ = (uint32_t)cb;
    int rc = ensure_capacity(slots_end_, cb);
    if (rc) return rc;
    if (ns > scene_cap_) {
        if (d_scenes_) cudaFree(d_scenes_);
        if (d_params_) cudaFree(d_params_);
        if (h_params_) cudaFreeHost(h_params_);
        scene_cap_ = std::max<uint64_t>(ns, scene_cap_ * 2);
        ENG_CK(cudaMalloc((void**)&d_scenes_, scene_cap_ * sizeof(DevScene)), "scene table");
        ENG_CK(cudaMalloc((void**)&d_params_, scene_cap_ * sizeof(DevParams)), "param table");
        ENG_CK(cudaMallocHost((void**)&h_params_, scene_cap_ * sizeof(DevParams)), "param staging");
        graph_dirty_ = true;
    }
    if (ns > tile_first_cap_) {
        if (d_tile_first_) cudaFree(d_tile_first_);
        tile_first_cap_ = std::max<uint64_t>(ns, tile_first_cap_ * 2);
        ENG_CK(cudaMalloc((void**)&d_tile_first_, tile_first_cap_ * sizeof(uint32_t)), "tile offsets");
    }
    if (ns > pend_cap_) {
        if (pend_) cudaFree(pend_);
        pend_cap_ = std::max<uint64_t>(ns, pend_cap_ * 2);
        ENG_CK(cudaMalloc((void**)&pend_, pend_cap_ * sizeof(uint32_t)), "pending flags");
        graph_dirty_ = true;
    }
    if (ns) ENG_CK(cudaMemcpyAsync(pend_, h_pend.data(), ns * sizeof(uint32_t), cudaMemcpyHostToDevice, stream_),
                   "pending flags upload");
    if (ntiles_ > tile_cap_) {
        if (d_tiles_) cudaFree(d_tiles_);
        tile_cap_ = std::max<uint64_t>(ntiles_, tile_cap_ * 2);
        ENG_CK(cudaMalloc((void**)&d_tiles_, tile_cap_ * sizeof(uint4)), "tile table");
        graph_dirty_ = true;
    }
    if (ns) ENG_CK(cudaMemcpyAsync(d_scenes_, h_scenes_.data(), ns * sizeof(DevScene), cudaMemcpyHostToDevice, stream_), "scene upload");
    if (ns) {
        ENG_CK(cudaMemcpyAsync(d_tile_first_, h_tile_first_.data(), ns * sizeof(uint32_t), cudaMemcpyHostToDevice,
                               stream_), "tile offsets upload");
        ENG_CK(launch_build_tiles(d_scenes_, d_tile_first_, (uint32_t)ns, exec_.tile, d_tiles_, stream_),
               "tile table");
    }
    ENG_CK(cudaStreamSynchronize(stream_), "layout sync");
    layout_dirty_ = false;
    params_dirty_ = true;
    graph_dirty_ = true;
    return ENG_OK;
}

int Engine::upload_params() {
    const size_t ns = scenes_.size();
    // The pinned staging buffer is reused: wait until the previous copy drained.
    ENG_CK(cudaStreamSynchronize(stream_), "param sync");
    bool all_defer = true;
    for (size_t k = 0; k < ns; ++k) {
        h_params_[k] = scenes_[k].dp;
        if (scene_defers(scenes_[k])) h_params_[k].flags |= SPH_FLAG_DEFER_XSPH;
        else all_defer = false;
    }
    if (all_defer != all_defer_) { all_defer_ = all_defer; graph_dirty_ = true; }
    if (ns) ENG_CK(cudaMemcpyAsync(d_params_, h_params_, ns * sizeof(DevParams), cudaMemcpyHostToDevice, stream_), "param upload");
    params_dirty_ = false;
    return ENG_OK;
}

StepArgs Engine::args() const {
    StepArgs a;
    a.params = d_params_;
    a.scenes = d_scenes_;
    a.tiles = d_tiles_;
    a.ntiles = ntiles_;
    a.particles = (uint32_t)total_particles();
    a.total_cells = total_cells_;
    a.P0 = P0_; a.V0 = V0_; a.A0 = A0_;
    a.P1 = P1_; a.V1 = V1_; a.A1 = A1_;
    a.V2 = V2_; a.S = S_; a.N = N_;
    a.Vc = Vc_; a.okey = okey_; a.pend = pend_;
    a.count = count_; a.start = start_; a.scan_sums = scan_sums_;
    a.scan_first = 0u;
    a.scan_cells = 0u;   // all cells
    a.scan_zeroes_counts = 1u;
    a.scan_spin_limit = scan_spin_limit_;
    a.scan_withhold = scan_withhold_ ? 1u : 0u;
    a.key = key_; a.slot = slot_; a.tmp = tmp_; a.perm = perm_;
    a.status = status_;
    a.mask = mask_;
    a.mask_stride = pcap_;
    a.maxdisp = scal_;
    a.block = exec_.tile;
    a.tile_ctr = exec_.persistent ? scal_ + 4 : nullptr;
    a.grid_nbr = exec_.persistent ? std::min<uint32_t>(a.ntiles, (uint32_t)sm_count_ * exec_.persistent) : a.ntiles;
    a.variant = exec_.variant;
    a.any_tension = any_tension_ ? 1u : 0u;
    a.skin_masks = all_defer_ ? 0u : 1u;
    a.dbg_nbr = debug_ ? dbg_nbr_ : nullptr;
    a.dbg_forces = debug_ ? dbg_forces_ : nullptr;
    return a;
}

// Record (or launch) the two halves of a substep on the stream.  The prefix
// (sort and density, with any pending XSPH update) ends where a state read
// needs it; the suffix is the rest (normals, forces and integrator, and the
// XSPH pass of scenes that do not defer it).
int Engine::launch_prefix(bool profile) { return launch_prefix_args(args(), profile, !hashed_); }

// The hash of the current positions, for when no force pass produced it (the
// first substep, or after the state, the layout or the parameters changed).
int Engine::launch_hash_standalone(const StepArgs& a) {
    ENG_CK(cudaMemsetAsync(count_, 0, (size_t)total_cells_ * sizeof(uint32_t), stream_), "memset counts");
    ENG_CK(launch_hash(a, stream_), "hash");
    return ENG_OK;
}

// The substep up to the density pass.  The hash normally comes from the
// previous substep's force pass; `hash` runs it here instead (the captured
// prefix graph never contains it).
int Engine::launch_prefix_args(const StepArgs& a, bool profile, bool hash) {
    cudaStream_t st = stream_;
    auto mark = [&](int i) { if (profile) cudaEventRecord(ev_[i], st); };
    mark(0);
    ENG_CK(cudaMemsetAsync(scal_, 0, 8 * sizeof(uint32_t), st), "memset substep scalars");
    if (hash) { int rc = launch_hash_standalone(a); if (rc) return rc; }
    mark(1);
    ENG_CK(launch_scan(a, st), "scan");
    mark(2);
    ENG_CK(launch_sort(a, st), "sort");
    mark(3);
    ENG_CK(launch_density(a, st), "density");
    mark(4);
    return ENG_OK;
}

int Engine::launch_suffix(bool profile) { return launch_suffix_args(args(), profile); }

int Engine::launch_suffix_args(const StepArgs& a, bool profile) {
    cudaStream_t st = stream_;
    auto mark = [&](int i) { if (profile) cudaEventRecord(ev_[i], st); };
    if (any_tension_) ENG_CK(launch_normals(a, st), "normals");
    mark(5);
    // the force pass hashes its output for the next substep, adding into the
    // counts that this substep's scan left at zero
    ENG_CK(launch_force(a, st), "force");
    mark(6);
    if (!all_defer_) ENG_CK(launch_xsph(a, st), "xsph");
    mark(7);
    return ENG_OK;
}

int Engine::read_status() {
    ENG_CK(cudaMemcpyAsync(h_status_, status_, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_), "status read");
    ENG_CK(cudaStreamSynchronize(stream_), "step sync");
    const uint32_t st = *h_status_;
    if (st) {
        hashed_ = false;   // hash the state afresh before the next substep
        ENG_CK(cudaMemsetAsync(status_, 0, sizeof(uint32_t), stream_), "status reset");
        if (st & SPH_STATUS_CELL_OVERFLOW)
            return fail(ENG_ECELL, "a grid cell held more than 8192 particles");
        if (st & SPH_STATUS_NONFINITE) return fail(ENG_ENAN, "non-finite particle position");
        if (st & SPH_STATUS_SCAN_TIMEOUT) return fail(ENG_ETIMEOUT, "cell scan: a look-back wait ran out");
    }
    return ENG_OK;
}

// The passes an export ran ahead (get_state) are undone: the state goes back
// to the prefix's gathered copies, and the cell counts, tile counters and
// hash that the force pass produced are cleared; the prefix itself stays
// valid.  Its status word (gate_) is dropped with it.
int Engine::settle() {
    if (!ahead_) return ENG_OK;
    ahead_ = false;
    ++ahead_undone_;
    if (++ahead_misses_ >= 2u) {
        ahead_skip_ = 16u;
        ahead_misses_ = 1u;   // one more miss after the pause pauses again
    }
    cudaSetDevice(device_);
    const Scene& s = scenes_.front();
    ENG_CK(launch_undo_ahead(args(), s.tile_first, s.tile_count, stream_), "undo");
    ENG_CK(cudaMemsetAsync(count_, 0, (size_t)total_cells_ * sizeof(uint32_t), stream_), "memset counts");
    ENG_CK(cudaMemsetAsync(scal_, 0, 8 * sizeof(uint32_t), stream_), "memset substep scalars");
    hashed_ = false;
    // an export that follows waits for this event before it packs the state
    ENG_CK(cudaEventRecord(suffix_ev_, stream_), "undo event");
    return ENG_OK;
}

// Layout, parameters and (in graph mode) the two captured graphs up to date.
int Engine::prepare() {
    if (!layout_dirty_ && !params_dirty_ && !graph_dirty_ && exec_pre_ && exec_suf_ && exec_full_) return ENG_OK;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = prepare_work();
    prep_seconds_ += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int Engine::prepare_work() {
    if (layout_dirty_ || params_dirty_) hashed_ = false;
    if (layout_dirty_) { int rc = rebuild_layout(); if (rc) return rc; }
    if (params_dirty_) { int rc = upload_params(); if (rc) return rc; }
    const bool graph = use_graph_ && !profiling_;
    if (graph && (graph_dirty_ || !exec_pre_ || !exec_suf_ || !exec_full_)) {
        // Re-capture; when only launch sizes and arguments changed (scenes
        // joined or left), update the instantiated graphs in place, which is
        // much cheaper than instantiating again.
        cudaGraph_t* graphs[] = {&graph_pre_, &graph_suf_, &graph_full_};
        cudaGraphExec_t* execs[] = {&exec_pre_, &exec_suf_, &exec_full_};
        for (int part = 0; part < 3; ++part) {
            cudaGraph_t& gref = *graphs[part];
            cudaGraphExec_t& eref = *execs[part];
            ENG_CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "begin capture");
            int rc = part == 1 ? ENG_OK : launch_prefix_args(args(), false, false);
            if (rc == ENG_OK && part != 0) rc = launch_suffix(false);
            cudaGraph_t g = nullptr;
            cudaError_t ce = cudaStreamEndCapture(stream_, &g);
            if (rc) { if (g) cudaGraphDestroy(g); return rc; }
            ENG_CK(ce, "end capture");
            bool updated = false;
            if (eref) {
                cudaGraphExecUpdateResultInfo info;
                updated = cudaGraphExecUpdate(eref, g, &info) == cudaSuccess;
                if (!updated) {
                    cudaGetLastError();   // the update's error is not sticky; instantiate instead
                    cudaGraphExecDestroy(eref);
                    eref = nullptr;
                }
            }
            if (gref) cudaGraphDestroy(gref);
            gref = g;
            if (!updated) ENG_CK(cudaGraphInstantiate(&eref, g, 0), "graph instantiate");
        }
        graph_dirty_ = false;
    }
    return ENG_OK;
}

int Engine::step(uint32_t substeps, bool sync) {
    cudaSetDevice(device_);
    if (scenes_.empty()) return ENG_OK;
    // no substeps: bring the layout, parameters and graphs up to date only
    // (a caller can then time substeps without the host work of a change)
    if (substeps == 0) {
        if (layout_dirty_ || params_dirty_) prefix_valid_ = false;
        return prepare();
    }
    // The passes an export ran ahead are this step's first substep when the
    // layout and parameters are those they ran with; their status word joins
    // this step's (the export found it clear).
    bool taken = false;
    if (ahead_) {
        if (!layout_dirty_ && !params_dirty_ && prefix_valid_) {
            ahead_ = false;
            ahead_misses_ = 0u;
            ++ahead_taken_;
            taken = true;
            ENG_CK(cudaMemcpyAsync(status_, gate_, sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream_),
                   "status merge");
        } else if (const int rc = settle()) {
            return rc;
        }
    }
    if (layout_dirty_ || params_dirty_) prefix_valid_ = false;
    int rc = prepare();
    if (rc) return rc;
    const bool graph = use_graph_ && !profiling_;
    eager_prefix_ = false;
    for (uint32_t s = 0; s < substeps; ++s) {
        if (s == 0 && taken) {
            // normals and forces ran ahead; nothing to launch
        } else if (graph) {
            if (!prefix_valid_) {
                if (!hashed_) { rc = launch_hash_standalone(args()); if (rc) return rc; }
                ENG_CK(cudaGraphLaunch(exec_full_, stream_), "graph launch");   // prefix and suffix
            } else {
                ENG_CK(cudaGraphLaunch(exec_suf_, stream_), "graph launch");
            }
        } else if (profiling_) {
            // a prefix computed for a state read is recomputed (same values) so
            // that every pass of the substep is timed
            rc = launch_prefix(true);
            if (rc) return rc;
            rc = launch_suffix(true);
            if (rc) return rc;
            ENG_CK(cudaEventSynchronize(ev_[7]), "profile sync");
            for (int i = 0; i < 7; ++i) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev_[i], ev_[i + 1]);
                // pass i spans events i..i+1, except that pass 0 includes the memsets
                pass_ms_[i] += ms;
            }
            float tot = 0.f;
            cudaEventElapsedTime(&tot, ev_[0], ev_[7]);
            pass_ms_[7] += tot;
            prof_substeps_++;
        } else {
            if (!prefix_valid_) { rc = launch_prefix(false); if (rc) return rc; }
            rc = launch_suffix(false);
            if (rc) return rc;
        }
        prefix_valid_ = false;
        hashed_ = true;
    }
    for (auto& s : scenes_) s.pending = scene_defers(s);
    stepped_ = true;
    if (!sync) return ENG_OK;
    if (graph && scenes_.size() == 1 && !debug_) {
        // A blocking step of a single system: read this step's status, then
        // launch the next substep's prefix, which the next step() or a state
        // read needs, and return once the status has arrived.  The GPU runs the
        // prefix while the caller takes the result.  Status bits the prefix
        // raises are read by the next call.  (Engines of many scenes, whose
        // layout changes between steps, compute it on demand instead, and so
        // does a system with debug taps, whose taps show the substep just run.)
        ENG_CK(cudaMemcpyAsync(h_status_, status_, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_), "status read");
        ENG_CK(cudaEventRecord(suffix_ev_, stream_), "step event");
        ENG_CK(cudaGraphLaunch(exec_pre_, stream_), "graph launch");
        prefix_valid_ = true;
        eager_prefix_ = true;
        hashed_ = false;   // the prefix's scan consumed the counts
        ENG_CK(cudaEventSynchronize(suffix_ev_), "step sync");
        if (*h_status_) {
            prefix_valid_ = false;
            eager_prefix_ = false;
            return read_status();   // waits for the prefix, reports and clears the bits
        }
        return ENG_OK;
    }
    return read_status();
}

// Run the next substep's prefix once, for reads of scenes whose XSPH update
// is pending: its density pass computes the updated velocities (Vc); the next
// step() starts from the suffix, so the work is not repeated.  With
// wait = false the caller reads the status word (read_status) afterwards and
// clears prefix_valid_ if it reports an error.
int Engine::ensure_prefix(bool wait) {
    if (layout_dirty_ || params_dirty_) prefix_valid_ = false;
    if (prefix_valid_) return ENG_OK;
    eager_prefix_ = false;
    int rc = prepare();
    if (rc) return rc;
    if (use_graph_ && !profiling_) {
        if (!hashed_) { rc = launch_hash_standalone(args()); if (rc) return rc; }
        ENG_CK(cudaGraphLaunch(exec_pre_, stream_), "graph launch");
    } else { rc = launch_prefix(false); if (rc) return rc; }
    // The scan consumed the counts: a prefix that runs again before the next
    // force pass (a parameter change, a profiled substep) hashes afresh.
    hashed_ = false;
    if (wait) {
        rc = read_status();
        if (rc) return rc;
    }
    prefix_valid_ = true;
    return ENG_OK;
}

// The prefix for one scene only (its tiles; every scene's cells are scanned,
// the others hold no particles then): a read of one scene of many costs that
// scene's share.  Scene-local, so its values equal a full prefix's; the full
// prefix is not valid afterwards.
int Engine::prefix_scene(const Scene& sc, bool wait) {
    int rc = prepare();
    if (rc) return rc;
    StepArgs a = args();
    a.tiles = d_tiles_ + sc.tile_first;
    a.ntiles = sc.tile_count;
    a.particles = sc.n;
    a.grid_nbr = sc.tile_count;
    a.tile_ctr = nullptr;
    a.scan_zeroes_counts = 0u;   // keep the counts for the full prefix that follows
    if (hashed_) {
        // Only this scene's cells hold counts that matter here: scan its own
        // range (cell starts relative to its first cell, as a full scan
        // gives them), not the cells of every live scene.  Without a fresh
        // hash the standalone hash below clears all counts, so the full range
        // is scanned as before.
        a.scan_first = cell_base_[sc.table_index];
        a.scan_cells = sc.dp.ncells + 1u;
    }
    rc = launch_prefix_args(a, false, !hashed_);
    if (rc) return rc;
    prefix_valid_ = false;
    return wait ? read_status() : ENG_OK;
}

// Write a pending XSPH update into the state (V0) and clear it.  A fresh
// prefix computes the same velocities from the updated state, so the prefix
// stays valid.
int Engine::materialize(Scene& s) {
    if (!s.pending) return ENG_OK;
    int rc = ensure_prefix();
    if (rc) return rc;
    const StepArgs a = args();
    ENG_CK(launch_unsort_vel(a, s.tile_first, s.tile_count, s.part_base, s.n, nullptr, V0_, true, stream_),
           "materialize");
    ENG_CK(cudaStreamSynchronize(stream_), "materialize sync");
    s.pending = false;
    return ENG_OK;
}

int Engine::materialize_all() {
    for (auto& s : scenes_) {
        int rc = materialize(s);
        if (rc) return rc;
    }
    return ENG_OK;
}

int Engine::set_deferred_xsph(bool on) {
    if (on == defer_xsph_) return ENG_OK;
    if (const int rc = settle()) return rc;
    if (!on) { int rc = materialize_all(); if (rc) return rc; }
    defer_xsph_ = on;
    params_dirty_ = true;
    prefix_valid_ = false;
    return ENG_OK;
}

int Engine::sync() {
    cudaSetDevice(device_);
    return read_status();
}

int Engine::set_profiling(bool on) {
    if (const int rc = settle()) return rc;
    profiling_ = on;
    for (double& v : pass_ms_) v = 0.0;
    prof_substeps_ = 0;
    return ENG_OK;
}

int Engine::timer_mark(int slot) {
    if (slot < 0 || slot >= 64) return fail(ENG_EINVAL, "timer slot out of range");
    cudaSetDevice(device_);
    // a region timed from here holds whole substeps: passes an export ran
    // ahead are undone (and run again inside the region)
    if (const int rc = settle()) return rc;
    if (!timers_[slot]) ENG_CK(cudaEventCreate(&timers_[slot]), "timer create");
    ENG_CK(cudaEventRecord(timers_[slot], stream_), "timer record");
    return ENG_OK;
}

int Engine::timer_elapsed(int a, int b, float* ms) {
    if (a < 0 || a >= 64 || b < 0 || b >= 64 || !timers_[a] || !timers_[b] || !ms)
        return fail(ENG_EINVAL, "timer slot not recorded");
    ENG_CK(cudaEventSynchronize(timers_[b]), "timer sync");
    ENG_CK(cudaEventElapsedTime(ms, timers_[a], timers_[b]), "timer elapsed");
    return ENG_OK;
}

int Engine::get_pass_times(double* ms_out, int cap, uint64_t* launches) {
    for (int i = 0; i < kPasses && i < cap; ++i) ms_out[i] = pass_ms_[i];
    if (launches) *launches = prof_substeps_;
    return ENG_OK;
}

void Engine::clear_pending(Scene& s) {
    s.pending = false;
    hashed_ = false;
    if (!layout_dirty_ && pend_ && s.table_index < pend_cap_) cudaMemsetAsync(pend_ + s.table_index, 0, sizeof(uint32_t), stream_);
    prefix_valid_ = false;
}

Scene* Engine::mscene(int id) {
    for (auto& s : scenes_) if (s.id == id) return &s;
    return nullptr;
}

int Engine::set_state(int id, const float* pos, const float* vel, uint32_t n, bool from_device) {
    cudaSetDevice(device_);
    if (const int rc = settle()) return rc;
    Scene* s = mscene(id);
    if (!s) return fail(ENG_EINVAL, "unknown scene id");
    if (n != s->n) return fail(ENG_EINVAL, "particle count mismatch");
    const float* dpos = pos;
    const float* dvel = vel;
    if (!from_device) {
        const size_t bytes = (size_t)n * 3 * sizeof(float);
        float* st = nullptr;
        int rc = staging(2 * bytes, &st);
        if (rc) return rc;
        ENG_CK(cudaMemcpyAsync(st, pos, bytes, cudaMemcpyHostToDevice, stream_), "state upload");
        dpos = st;
        dvel = nullptr;
        if (vel) {
            ENG_CK(cudaMemcpyAsync(st + (size_t)n * 3, vel, bytes, cudaMemcpyHostToDevice, stream_), "state upload");
            dvel = st + (size_t)n * 3;
        }
    }
    clear_pending(*s);
    ENG_CK(launch_unpack(dpos, dvel, n, s->part_base, P0_, V0_, A0_, S_, stream_), "unpack");
    ENG_CK(cudaStreamSynchronize(stream_), "upload sync");
    return ENG_OK;
}

int Engine::set_positions(int id, uint32_t first, const float* pos, uint32_t count) {
    cudaSetDevice(device_);
    if (const int rc = settle()) return rc;
    Scene* s = mscene(id);
    if (!s) return fail(ENG_EINVAL, "unknown scene id");
    if ((uint64_t)first + count > s->n) return fail(ENG_EINVAL, "range exceeds the scene's particle count");
    if (count == 0) return ENG_OK;
    // the other particles keep their velocities: apply a pending XSPH update first
    if (s->pending) { int rc = materialize(*s); if (rc) return rc; }
    prefix_valid_ = false;
    hashed_ = false;
    const size_t bytes = (size_t)count * 3 * sizeof(float);
    float* st = nullptr;
    int rc = staging(bytes, &st);
    if (rc) return rc;
    ENG_CK(cudaMemcpyAsync(st, pos, bytes, cudaMemcpyHostToDevice, stream_), "position upload");
    ENG_CK(launch_set_positions(st, count, s->part_base + first, P0_, stream_), "set positions");
    ENG_CK(cudaStreamSynchronize(stream_), "upload sync");
    return ENG_OK;
}

int Engine::generate_lattice(int id, const LatticeSpec& spec, uint32_t first) {
    cudaSetDevice(device_);
    if (const int rc = settle()) return rc;
    Scene* s = mscene(id);
    if (!s) return fail(ENG_EINVAL, "unknown scene id");
    const uint64_t n = (uint64_t)spec.nx * spec.ny * spec.nz;
    if (first + n > s->n) return fail(ENG_EINVAL, "lattice exceeds the scene's particle count");
    if (s->pending) { int rc = materialize(*s); if (rc) return rc; }
    prefix_valid_ = false;
    hashed_ = false;
    ENG_CK(launch_lattice(spec, s->part_base + first, P0_, V0_, A0_, S_, stream_), "lattice");
    return ENG_OK;
}

int Engine::get_state(int id, float* pos, float* colour, float* vel, uint32_t n, bool to_device) {
    cudaSetDevice(device_);
    if (const int rc = settle()) return rc;
    Scene* s = mscene(id);
    if (!s) return fail(ENG_EINVAL, "unknown scene id");
    if (n != s->n) return fail(ENG_EINVAL, "particle count mismatch");
    // A pending XSPH update: the next substep's prefix computes the updated
    // velocities (cell order), read back into state order; the state itself
    // is not changed, so reading never alters the trajectory.
    const bool pend = s->pending && vel;
    // one scene of several, and no full prefix at hand: that scene's prefix only
    auto run_prefix = [&](bool wait) {
        if (layout_dirty_ || params_dirty_) prefix_valid_ = false;
        return (prefix_valid_ || scenes_.size() == 1) ? ensure_prefix(wait) : prefix_scene(*s, wait);
    };
    if (pend && to_device) {
        int rc = run_prefix(true);
        if (rc) return rc;
    }
    if (to_device) {
        const StepArgs a = args();
        ENG_CK(launch_pack(P0_, V0_, n, s->part_base, s->dp.inv_rest_density, pos, colour, pend ? nullptr : vel,
                           stream_), "pack");
        if (pend) ENG_CK(launch_unsort_vel(a, s->tile_first, s->tile_count, s->part_base, s->n, vel, nullptr, false,
                                           stream_), "unsort");
        ENG_CK(cudaStreamSynchronize(stream_), "pack sync");
        return ENG_OK;
    }
    // (Writing registered host buffers directly from the pack kernel over the
    // host link measured 2x slower than packing into device memory and copying
    // with the copy engine, so exports always stage.)
    const size_t bytes = (size_t)n * 3 * sizeof(float);
    float* st = nullptr;
    int rc = staging(3 * bytes, &st);
    if (rc) return rc;
    float* dp = pos ? st : nullptr;
    float* dc = colour ? st + (size_t)n * 3 : nullptr;
    float* dv = vel ? st + (size_t)n * 6 : nullptr;
    if (eager_prefix_ && prefix_valid_ && !layout_dirty_ && !params_dirty_) {
        // The last blocking step left the next prefix running behind
        // suffix_ev_: the state it ended with (P0; V0 when no update is
        // pending) is packed and copied on the copy stream meanwhile, and a
        // pending update's velocities follow the prefix on the main stream.
        // Export ahead (set_export_ahead): the velocities cross the host link
        // on the copy stream while the main stream runs the next substep's
        // normal and force passes, with their own status word, which starts
        // failed when the prefix reported an error; they write the state
        // only after the pack has read it.
        bool ahead = pend && ahead_enabled_ && all_defer_ && use_graph_ && !profiling_ && !debug_ &&
                     scenes_.size() == 1;
        if (ahead && ahead_skip_ > 0) {
            --ahead_skip_;
            ahead = false;
        }
        ENG_CK(cudaStreamWaitEvent(copy_stream_, suffix_ev_, 0), "export wait");
        ENG_CK(launch_pack(P0_, V0_, n, s->part_base, s->dp.inv_rest_density, dp, dc, pend ? nullptr : dv,
                           copy_stream_), "pack");
        if (ahead) ENG_CK(cudaEventRecord(pack_ev_, copy_stream_), "pack event");
        if (pos) ENG_CK(cudaMemcpyAsync(pos, dp, bytes, cudaMemcpyDeviceToHost, copy_stream_), "download");
        if (colour) ENG_CK(cudaMemcpyAsync(colour, dc, bytes, cudaMemcpyDeviceToHost, copy_stream_), "download");
        if (vel && !pend) ENG_CK(cudaMemcpyAsync(vel, dv, bytes, cudaMemcpyDeviceToHost, copy_stream_), "download");
        if (pend) {
            const StepArgs a = args();
            ENG_CK(launch_unsort_vel(a, s->tile_first, s->tile_count, s->part_base, s->n, dv, nullptr, false, stream_,
                                     ahead ? gate_ : nullptr),
                   "unsort");
            if (ahead) {
                ENG_CK(cudaEventRecord(vel_ev_, stream_), "unsort event");
                ENG_CK(cudaStreamWaitEvent(copy_stream_, vel_ev_, 0), "export wait");
                ENG_CK(cudaMemcpyAsync(vel, dv, bytes, cudaMemcpyDeviceToHost, copy_stream_), "download");
                ENG_CK(cudaMemcpyAsync(h_status_, status_, sizeof(uint32_t), cudaMemcpyDeviceToHost, copy_stream_),
                       "status read");
                ENG_CK(cudaStreamWaitEvent(stream_, pack_ev_, 0), "ahead wait");
                StepArgs b = a;
                b.status = gate_;
                rc = launch_suffix_args(b, false);
                if (rc) return rc;
                ahead_ = true;
                ++ahead_started_;
            } else {
                ENG_CK(cudaMemcpyAsync(vel, dv, bytes, cudaMemcpyDeviceToHost, stream_), "download");
            }
        }
        const cudaError_t ce = cudaStreamSynchronize(copy_stream_);
        if (ce != cudaSuccess) return cuda_fail(ce, "download sync");
        if (ahead_) {
            if (*h_status_ == 0u) return ENG_OK;
            // the passes run ahead found their status word failed and did
            // nothing (they do not count as run): report the prefix's error
            ahead_ = false;
            --ahead_started_;
        }
        rc = read_status();   // the prefix's status; waits for the main stream too
        if (rc) { prefix_valid_ = false; eager_prefix_ = false; return rc; }
        return ENG_OK;
    }
    ENG_CK(launch_pack(P0_, V0_, n, s->part_base, s->dp.inv_rest_density, dp, dc, pend ? nullptr : dv, stream_),
           "pack");
    if (!pend) {
        if (pos) ENG_CK(cudaMemcpyAsync(pos, dp, bytes, cudaMemcpyDeviceToHost, stream_), "download");
        if (colour) ENG_CK(cudaMemcpyAsync(colour, dc, bytes, cudaMemcpyDeviceToHost, stream_), "download");
        if (vel) ENG_CK(cudaMemcpyAsync(vel, dv, bytes, cudaMemcpyDeviceToHost, stream_), "download");
        ENG_CK(cudaStreamSynchronize(stream_), "download sync");
        return ENG_OK;
    }
    // Positions and colours do not depend on the pending XSPH update (the
    // prefix reads P0 and does not write it): they cross the host link on the
    // copy stream while the prefix computes the velocities.
    ENG_CK(cudaEventRecord(copy_ev_, stream_), "export event");
    ENG_CK(cudaStreamWaitEvent(copy_stream_, copy_ev_, 0), "export wait");
    if (pos) ENG_CK(cudaMemcpyAsync(pos, dp, bytes, cudaMemcpyDeviceToHost, copy_stream_), "download");
    if (colour) ENG_CK(cudaMemcpyAsync(colour, dc, bytes, cudaMemcpyDeviceToHost, copy_stream_), "download");
    rc = run_prefix(false);
    if (rc == ENG_OK) {
        const StepArgs a = args();
        ENG_CK(launch_unsort_vel(a, s->tile_first, s->tile_count, s->part_base, s->n, dv, nullptr, false, stream_),
               "unsort");
        ENG_CK(cudaMemcpyAsync(vel, dv, bytes, cudaMemcpyDeviceToHost, stream_), "download");
    }
    const cudaError_t ce = cudaStreamSynchronize(copy_stream_);
    if (rc) return rc;
    if (ce != cudaSuccess) return cuda_fail(ce, "download sync");
    rc = read_status();   // the prefix's status; waits for the velocity copy too
    if (rc) { prefix_valid_ = false; return rc; }
    return ENG_OK;
}

int Engine::save_state(int id, float4* host, uint32_t n) {
    cudaSetDevice(device_);
    if (const int rc = settle()) return rc;
    Scene* s = mscene(id);
    if (!s) return fail(ENG_EINVAL, "unknown scene id");
    if (n != s->n) return fail(ENG_EINVAL, "particle count mismatch");
    if (n == 0) return ENG_OK;
    // the snapshot holds a final state: apply a pending XSPH update (the
    // values are those the next substep would use, so the run continues alike)
    if (s->pending) { int rc = materialize(*s); if (rc) return rc; }
    const size_t bytes = (size_t)n * sizeof(float4);
    ENG_CK(cudaMemcpyAsync(host, P0_ + s->part_base, bytes, cudaMemcpyDeviceToHost, stream_), "snapshot");
    ENG_CK(cudaMemcpyAsync(host + n, V0_ + s->part_base, bytes, cudaMemcpyDeviceToHost, stream_), "snapshot");
    ENG_CK(cudaMemcpyAsync(host + 2 * (size_t)n, A0_ + s->part_base, bytes, cudaMemcpyDeviceToHost, stream_),
           "snapshot");
    ENG_CK(cudaStreamSynchronize(stream_), "snapshot sync");
    return ENG_OK;
}

int Engine::load_state(int id, const float4* host, uint32_t n) {
    cudaSetDevice(device_);
    if (const int rc = settle()) return rc;
    Scene* s = mscene(id);
    if (!s) return fail(ENG_EINVAL, "unknown scene id");
    if (n != s->n) return fail(ENG_EINVAL, "particle count mismatch");
    if (n == 0) return ENG_OK;
    clear_pending(*s);
    const size_t bytes = (size_t)n * sizeof(float4);
    ENG_CK(cudaMemcpyAsync(P0_ + s->part_base, host, bytes, cudaMemcpyHostToDevice, stream_), "restore");
    ENG_CK(cudaMemcpyAsync(V0_ + s->part_base, host + n, bytes, cudaMemcpyHostToDevice, stream_), "restore");
    ENG_CK(cudaMemcpyAsync(A0_ + s->part_base, host + 2 * (size_t)n, bytes, cudaMemcpyHostToDevice, stream_),
           "restore");
    ENG_CK(cudaMemsetAsync(S_ + s->part_base, 0, bytes, stream_), "restore");
    ENG_CK(cudaStreamSynchronize(stream_), "restore sync");
    return ENG_OK;
}

int Engine::debug_enable(bool on) {
    if (on == debug_) return ENG_OK;
    if (const int rc = settle()) return rc;
    // debug taps show each substep's own passes: XSPH runs in every substep
    if (on) { int rc = materialize_all(); if (rc) return rc; }
    debug_ = on;
    graph_dirty_ = true;
    params_dirty_ = true;
    prefix_valid_ = false;
    if (on && pcap_) {
        ENG_CK(cudaMalloc((void**)&dbg_nbr_, pcap_ * sizeof(uint32_t)), "debug alloc");
        ENG_CK(cudaMalloc((void**)&dbg_forces_, pcap_ * 4 * sizeof(float4)), "debug alloc");
    }
    return ENG_OK;
}

int Engine::debug_get(int id, int field, void* host, uint64_t count) {
    cudaSetDevice(device_);
    if (const int rc = settle()) return rc;
    ENG_CK(cudaStreamSynchronize(stream_), "debug sync");
    const Scene* s = scene(id);
    if (!s) return fail(ENG_EINVAL, "unknown scene id");
    if (!stepped_) return fail(ENG_EINVAL, "no substep has run yet");
    size_t k = 0;
    for (; k < scenes_.size(); ++k) if (scenes_[k].id == id) break;
    const uint32_t n = s->n, nc = s->dp.ncells, cb = cell_base_[k], pb = s->part_base;
    auto need = [&](uint64_t c) { return count >= c; };
    switch (field) {
        case F_HASH: {
            if (!need(n)) return fail(ENG_EINVAL, "buffer too small");
            uint32_t* tmp = nullptr;
            ENG_CK(cudaMalloc((void**)&tmp, n * sizeof(uint32_t)), "debug alloc");
            ENG_CK(launch_sorted_keys(d_params_ + s->table_index, P1_, n, pb, tmp, stream_), "sorted keys");
            ENG_CK(cudaMemcpyAsync(host, tmp, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_), "debug copy");
            ENG_CK(cudaStreamSynchronize(stream_), "debug sync");
            cudaFree(tmp);
            return ENG_OK;
        }
        case F_PERM: {
            if (!need(n)) return fail(ENG_EINVAL, "buffer too small");
            uint32_t* out = (uint32_t*)host;
            ENG_CK(cudaMemcpy(out, perm_ + pb, n * sizeof(uint32_t), cudaMemcpyDeviceToHost), "debug copy");
            for (uint32_t i = 0; i < n; ++i) out[i] -= pb;
            return ENG_OK;
        }
        case F_CELLSTART:
        case F_CELLOCC: {
            if (!need(nc)) return fail(ENG_EINVAL, "buffer too small");
            std::vector<uint32_t> st(nc + 1);
            ENG_CK(cudaMemcpy(st.data(), start_ + cb, (nc + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost), "debug copy");
            uint32_t* out = (uint32_t*)host;
            for (uint32_t c = 0; c < nc; ++c) out[c] = (field == F_CELLSTART) ? st[c] - st[0] : st[c + 1] - st[c];
            return ENG_OK;
        }
        case F_NBRCOUNT: {
            if (!debug_ || !dbg_nbr_) return fail(ENG_EINVAL, "debug taps are not enabled");
            if (!need(n)) return fail(ENG_EINVAL, "buffer too small");
            ENG_CK(cudaMemcpy(host, dbg_nbr_ + pb, n * sizeof(uint32_t), cudaMemcpyDeviceToHost), "debug copy");
            return ENG_OK;
        }
        case F_DENSITY:
        case F_PRESSURE:
        case F_SOUNDSPEED: {
            if (!need(n)) return fail(ENG_EINVAL, "buffer too small");
            std::vector<float4> v(n);
            ENG_CK(cudaMemcpy(v.data(), S_ + pb, n * sizeof(float4), cudaMemcpyDeviceToHost), "debug copy");
            float* out = (float*)host;
            for (uint32_t i = 0; i < n; ++i)
                out[i] = field == F_DENSITY ? v[i].x : field == F_PRESSURE ? v[i].y : v[i].z;
            return ENG_OK;
        }
        case F_FPRESSURE:
        case F_FTENSION:
        case F_FADHESION:
        case F_FVISCOSITY: {
            if (!debug_ || !dbg_forces_) return fail(ENG_EINVAL, "debug taps are not enabled");
            if (!need(3ull * n)) return fail(ENG_EINVAL, "buffer too small");
            std::vector<float4> v((size_t)n * 4);
            ENG_CK(cudaMemcpy(v.data(), dbg_forces_ + 4 * (size_t)pb, (size_t)n * 4 * sizeof(float4), cudaMemcpyDeviceToHost), "debug copy");
            const int c = field - F_FPRESSURE;
            float* out = (float*)host;
            for (uint32_t i = 0; i < n; ++i) {
                const float4 f = v[4 * (size_t)i + c];
                out[3 * i] = f.x; out[3 * i + 1] = f.y; out[3 * i + 2] = f.z;
            }
            return ENG_OK;
        }
        case F_NORMAL:
        case F_POS_SORTED:
        case F_ACC:
        case F_VEL_INT: {
            if (!need(3ull * n)) return fail(ENG_EINVAL, "buffer too small");
            const float4* src = field == F_NORMAL ? N_ : field == F_POS_SORTED ? P1_ : field == F_ACC ? A0_ : V2_;
            std::vector<float4> v(n);
            ENG_CK(cudaMemcpy(v.data(), src + pb, n * sizeof(float4), cudaMemcpyDeviceToHost), "debug copy");
            float* out = (float*)host;
            for (uint32_t i = 0; i < n; ++i) { out[3 * i] = v[i].x; out[3 * i + 1] = v[i].y; out[3 * i + 2] = v[i].z; }
            return ENG_OK;
        }
        default:
            return fail(ENG_EINVAL, "unknown debug field");
    }
}

}  // namespace sph
