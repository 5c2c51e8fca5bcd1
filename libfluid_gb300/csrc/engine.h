// Host-side engine: device arenas, scene table, tile list and the captured
// substep.  One Engine drives any number of independent scenes with one
// launch per pass; the plain FluidSystem drop-in is an Engine with one scene.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <map>
#include <string>
#include <vector>
#include "sph_types.h"
#include "sph_kernels.h"

namespace sph {

// User-facing parameters of one scene: the values FluidParams' setters take
// (fluidparams.cuh:103-117) plus the generalised domain and gravity.
struct SceneConfig {
    int box_mode = 0;                 // 0: unit cube with res cells per axis (the reference); 1: box lx,ly,lz, cell h
    uint32_t res = 1;
    float lx = 1.f, ly = 1.f, lz = 1.f, h = 1.f;
    float rest_density = 1.f, gas_constant = 1.f, gamma = 1.f, mass = 1.f, particle_size = 1.f;
    float xsph = 0.5f, surface_tension = 1.f, viscosity = 0.1f, adhesion = 1.f, vdamp = 1.f;
    float vel_limit = 5.f, acc_limit = 150.f, dt = 0.01f;
    float gravity[3] = {0.f, -9.8f, 0.f};
    float skin = 0.f;                 // neighbour-mask skin in units of h (0: engine default)
    int boundary = 0;                 // 0: the box; 1: the sphere of radius min half extent about its centre
};

// Execution choices of the substep.  Defaults are the autotuner's choice
// (libfluid_gb300/autotune.py, recorded in libfluid_gb300/tuned.json) for the
// 1M dam break and the 256-scene batch alike.
struct ExecConfig {
    uint32_t tile = 128;              // particles per tile = threads per block (64, 128 or 256)
    uint32_t persistent = 0;          // 0: one block per tile; k > 0: k blocks per SM pull tiles
    float skin = SPH_SKIN_DEFAULT;    // neighbour-mask skin (units of h)
    uint32_t variant = SPH_VARIANT_DEFAULT;  // SPH_VARIANT_* bits
};

// Derive the device parameter block (FluidParams::setRes and setters,
// fluidparams.cu:51-213).  Returns false for an unusable domain.
bool derive_params(const SceneConfig& c, DevParams& out, std::string* err);

struct Scene {
    int id = -1;
    uint32_t part_base = 0, n = 0;
    SceneConfig cfg;
    DevParams dp{};
    // Its last substep's XSPH update is not yet applied to the state: the
    // next density pass applies it (deferred XSPH).
    bool pending = false;
    // position in the device scene table and its tiles, as of the last layout
    uint32_t table_index = 0, tile_first = 0, tile_count = 0;
};

enum { ENG_OK = 0, ENG_EINVAL = 1, ENG_ENOMEM = 2, ENG_ECUDA = 3, ENG_ENAN = 4, ENG_ETIMEOUT = 5, ENG_ECELL = 7 };

class Engine {
public:
    explicit Engine(int device = -1);
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    // Scene management (only between steps).
    int add_scene(const SceneConfig& cfg, uint32_t n, int* id_out);
    int remove_scene(int id);
    int set_config(int id, const SceneConfig& cfg);
    const Scene* scene(int id) const;
    size_t num_scenes() const { return scenes_.size(); }
    uint64_t total_particles() const;

    // State transfer (host packed xyz float32; device pointers allowed).
    int set_state(int id, const float* pos, const float* vel, uint32_t n, bool from_device = false);
    int set_positions(int id, uint32_t first, const float* pos, uint32_t count);
    int generate_lattice(int id, const LatticeSpec& spec, uint32_t first);
    int get_state(int id, float* pos, float* colour, float* vel, uint32_t n, bool to_device = false);
    // Exact state (3n float4 on the host: positions, velocities,
    // accelerations, in slot order, w lanes included) for snapshot/resume.
    int save_state(int id, float4* host, uint32_t n);
    int load_state(int id, const float4* host, uint32_t n);

    // Advance every live scene by `substeps` substeps (all with their own dt).
    // With substeps == 0, only bring the layout, parameters and captured
    // graphs up to date (nothing is launched).
    int step(uint32_t substeps, bool sync = true);
    int sync();

    // Debug taps (copy to host).  Valid after at least one substep.
    int debug_enable(bool on);
    enum Field { F_HASH = 0, F_PERM, F_CELLSTART, F_CELLOCC, F_NBRCOUNT, F_DENSITY, F_PRESSURE, F_SOUNDSPEED,
                 F_FPRESSURE, F_FTENSION, F_FADHESION, F_FVISCOSITY, F_NORMAL, F_POS_SORTED, F_ACC, F_VEL_INT };
    int debug_get(int id, int field, void* host, uint64_t count);

    // XSPH schedule.  Deferred (the default): a substep ends after the
    // integrator and its XSPH update is applied by the next substep's density
    // pass, fused into that walk; reading a scene's state (export, snapshot)
    // first runs the next substep's sort and density pass, whose result the
    // next step reuses, so reading never changes the trajectory.  Otherwise
    // (and always with debug taps on, or for grids above SPH_OKEY_MAX_DIM cells
    // per axis) every substep runs its own XSPH pass, as the reference does.
    int set_deferred_xsph(bool on);
    bool deferred_xsph() const { return defer_xsph_; }

    // Test control of the cell scan's look-back waits: spin_limit polls per
    // wait (0: the default), and with `withhold` no block takes the first
    // tile, so every wait that reaches it runs out and the step reports
    // ENG_ETIMEOUT with the state as it was before the failed substep.
    int set_scan_fault(uint32_t spin_limit, bool withhold) {
        const int rc = settle();
        scan_spin_limit_ = spin_limit;
        scan_withhold_ = withhold;
        graph_dirty_ = true;
        prefix_valid_ = false;
        return rc;
    }

    // Options.
    int set_use_graph(bool on) {
        const int rc = settle();
        use_graph_ = on;
        graph_dirty_ = true;
        return rc;
    }
    // Export ahead (on by default).  A blocking export of a single scene
    // whose velocities wait for the XSPH update (deferred XSPH) starts the
    // next substep's normal and force passes once that update is computed,
    // so that they run while the velocities cross the host link.  The next
    // step() takes them as its first substep when nothing changed in
    // between; every other call first undoes them exactly (settle()), so
    // results do not depend on this option.
    int set_export_ahead(bool on) {
        const int rc = settle();
        ahead_enabled_ = on;
        return rc;
    }
    bool export_ahead() const { return ahead_enabled_; }
    // Exports that ran passes ahead, and how many of those a step took and
    // how many were undone.
    void export_ahead_stats(uint64_t out[3]) const {
        out[0] = ahead_started_;
        out[1] = ahead_taken_;
        out[2] = ahead_undone_;
    }
    int set_exec(const ExecConfig& e);
    const ExecConfig& exec() const { return exec_; }
    int sm_count() const { return sm_count_; }
    cudaStream_t stream() const { return stream_; }
    double prep_seconds() const { return prep_seconds_; }
    const std::string& last_error() const { return err_; }
    int device() const { return device_; }

    // Per-pass timing with CUDA events (profiling runs; disables the graph).
    int set_profiling(bool on);
    int get_pass_times(double* ms_out, int cap, uint64_t* launches);
    static const char* pass_name(int i);
    static constexpr int kPasses = 8;

    // Device timers on the engine's stream.
    int timer_mark(int slot);
    int timer_elapsed(int a, int b, float* ms);

    // Byte footprint of the arenas (for admission control).
    static uint64_t bytes_per_particle();
    static uint64_t bytes_per_cell();
    uint64_t device_bytes() const { return dev_bytes_; }
    // Cap on the arena footprint (0 = none): growth beyond it fails with ENG_ENOMEM.
    void set_byte_limit(uint64_t bytes) { byte_limit_ = bytes; }
    // Grow the arenas to at least this many particle slots and cells now.
    int reserve(uint64_t parts, uint64_t cells) {
        if (const int rc = settle()) return rc;
        return ensure_capacity(parts, cells);
    }

private:
    int fail(int code, const std::string& msg);
    int cuda_fail(cudaError_t e, const char* what);
    int ensure_capacity(uint64_t parts, uint64_t cells);
    int rebuild_layout();
    int upload_params();
    int launch_prefix(bool profile);   // [memset, hash], scan, sort, density
    int launch_prefix_args(const StepArgs& a, bool profile, bool hash);
    int launch_hash_standalone(const StepArgs& a);
    int prefix_scene(const Scene& s, bool wait = true);  // the prefix over one scene's tiles
    int launch_suffix(bool profile);   // normals, force + integrator, [XSPH]
    int launch_suffix_args(const StepArgs& a, bool profile);
    // Undo the passes an export ran ahead, if any (see set_export_ahead):
    // every entry point that reads or changes the state, changes how it is
    // stepped, or marks a timer calls this first; step() takes the passes
    // instead, and sync() only waits for them.
    int settle();
    int ensure_prefix(bool wait = true);   // the next substep's prefix, computed once
    int materialize(Scene& s);         // apply a pending XSPH update to the state
    int materialize_all();
    void clear_pending(Scene& s);      // state replaced: nothing pending
    Scene* mscene(int id);
    bool scene_defers(const Scene& s) const {
        return defer_xsph_ && !debug_ && s.dp.gx <= SPH_OKEY_MAX_DIM && s.dp.gy <= SPH_OKEY_MAX_DIM &&
               s.dp.gz <= SPH_OKEY_MAX_DIM;
    }
    int prepare();
    int prepare_work();                     // layout, params and graphs up to date
    int read_status();
    double prep_seconds_ = 0.0;        // host time spent in prepare() (layout, parameters, graphs)
    void free_all();
    uint32_t alloc_slots(uint32_t n);
    void free_slots(uint32_t base, uint32_t n);
    int staging(size_t bytes, float** out);
    StepArgs args() const;

    int device_ = 0;
    cudaStream_t stream_ = nullptr;
    cudaStream_t copy_stream_ = nullptr;   // exports: copies that overlap the prefix
    cudaEvent_t copy_ev_ = nullptr;
    cudaEvent_t suffix_ev_ = nullptr;      // the last blocking step's suffix (and status read) done
    cudaEvent_t pack_ev_ = nullptr;        // an export's pack of the state done (export ahead)
    cudaEvent_t vel_ev_ = nullptr;         // an export's velocities unsorted (export ahead)
    std::string err_;
    std::vector<Scene> scenes_;
    int next_id_ = 1;
    // free slot ranges: base -> length
    std::map<uint32_t, uint32_t> free_;
    uint64_t pcap_ = 0, ccap_ = 0, slots_end_ = 0;
    // device arenas
    float4 *P0_ = nullptr, *P1_ = nullptr, *V0_ = nullptr, *V1_ = nullptr, *V2_ = nullptr, *A0_ = nullptr,
           *A1_ = nullptr, *S_ = nullptr, *N_ = nullptr, *Vc_ = nullptr;
    uint32_t *okey_ = nullptr;         // packed cells of the last substep (state order)
    uint32_t *pend_ = nullptr;                      // per scene-table entry: XSPH update pending
    uint32_t *key_ = nullptr, *slot_ = nullptr, *tmp_ = nullptr, *perm_ = nullptr;
    uint32_t *count_ = nullptr, *start_ = nullptr, *scan_sums_ = nullptr, *status_ = nullptr;
    uint32_t *gate_ = nullptr;        // status word of the passes an export ran ahead (status_ + 1)
    uint32_t *mask_ = nullptr;        // SPH_MASK_ROWS neighbour-mask words per slot
    uint32_t *scal_ = nullptr;        // per-substep scalars: [0] displacement max, [4..7] tile counters
    ExecConfig exec_;
    int sm_count_ = 1;
    uint32_t* dbg_nbr_ = nullptr;
    float* stage_ = nullptr;           // device staging for packed xyz transfers
    size_t stage_bytes_ = 0;
    float4* dbg_forces_ = nullptr;
    DevParams* d_params_ = nullptr;
    DevScene* d_scenes_ = nullptr;
    uint4* d_tiles_ = nullptr;
    uint64_t scene_cap_ = 0, tile_cap_ = 0;
    uint64_t dev_bytes_ = 0;
    uint64_t byte_limit_ = 0;
    // host mirrors
    DevParams* h_params_ = nullptr;    // pinned
    uint32_t* h_status_ = nullptr;     // pinned
    std::vector<DevScene> h_scenes_;
    std::vector<uint32_t> h_tile_first_;   // per scene: its first tile (the tiles are built on the device)
    uint32_t ntiles_ = 0;
    uint32_t* d_tile_first_ = nullptr;
    uint64_t tile_first_cap_ = 0;
    std::vector<uint32_t> cell_base_;
    uint32_t total_cells_ = 0;
    bool any_tension_ = false;
    bool layout_dirty_ = true, params_dirty_ = true, graph_dirty_ = true;
    bool debug_ = false, use_graph_ = true, profiling_ = false;
    bool stepped_ = false;
    bool defer_xsph_ = true;
    bool all_defer_ = false;           // every scene defers: no XSPH pass in the substep
    uint64_t pend_cap_ = 0;
    uint32_t scan_spin_limit_ = 0;     // set_scan_fault
    bool scan_withhold_ = false;
    bool prefix_valid_ = false;        // the next substep's prefix has run (for a state read)
    bool eager_prefix_ = false;        // that prefix was launched by step() behind suffix_ev_
    bool ahead_enabled_ = true;        // set_export_ahead
    bool ahead_ = false;               // an export ran the next substep's suffix ahead; not yet taken
    // A caller whose next call rarely takes the passes (a time step that
    // changes every frame, reads after the export) would pay for them: after
    // two undone in a row the next 16 exports run nothing ahead, then one
    // tries again.
    uint32_t ahead_misses_ = 0, ahead_skip_ = 0;
    uint64_t ahead_started_ = 0, ahead_taken_ = 0, ahead_undone_ = 0;
    bool hashed_ = false;              // key, slot and cell counts describe the current P0 (the
                                       // last force pass hashed its output and no full prefix's scan
                                       // has consumed the counts since); else the prefix hashes
    // the substep captured as prefix, suffix, and both in one graph (one
    // launch per substep in a run of substeps)
    cudaGraph_t graph_pre_ = nullptr, graph_suf_ = nullptr, graph_full_ = nullptr;
    cudaGraphExec_t exec_pre_ = nullptr, exec_suf_ = nullptr, exec_full_ = nullptr;
    cudaEvent_t ev_[kPasses + 1] = {};
    cudaEvent_t timers_[64] = {};
    double pass_ms_[kPasses] = {};
    uint64_t prof_substeps_ = 0;
};

}  // namespace sph
