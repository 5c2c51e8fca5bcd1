/*
 * sph_c.h - C ABI of the GB300-native WCSPH step (libsph_gb300.so).
 *
 * This is the boundary under which NCCA/libfluid's FluidSystem
 * (libfluid/include/fluidsystem.h:16-126) is replaced.  Every entry point
 * names the reference member it stands for.  Plain pointers and sizes only:
 * positions, velocities and colours cross the boundary as packed float32 xyz
 * triples (the layout of std::vector<float3>), n particles = 3n floats.
 *
 * Errors: every function returns SPH_OK (0) or an SPH_E* code; the message
 * of the last failure on a handle is available from sph_last_error().  The
 * reference returns void and calls exit(0) on CUDA errors
 * (fluidparams.cu:222-227, fluidsystem.cu:253-258); this library never exits.
 *
 * Threading: a handle is used by one host thread at a time.  Each handle owns
 * a CUDA stream and its own parameter block in device memory, so any number
 * of handles coexist (the reference keeps one __constant__ block per process,
 * fluidparams.cu:6).
 */
#ifndef SPH_C_H
#define SPH_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum sph_status {
    SPH_OK = 0,
    SPH_EINVAL = 1,    /* bad argument or call order */
    SPH_ENOMEM = 2,    /* device allocation failed or budget exceeded */
    SPH_ECUDA = 3,     /* CUDA runtime error */
    SPH_ENAN = 4,      /* a non-finite particle position appeared */
    SPH_ETIMEOUT = 5,  /* a bounded wait ran out */
    SPH_ENOTINIT = 6,  /* advance/export before init (the reference silently returns) */
    SPH_ECELL = 7,     /* a grid cell held more than 8192 particles; the substep left them as they were */
    SPH_EBUSY = 8      /* request rejected: over capacity */
};

typedef struct sph_system sph_system;

/* ---- lifetime ---------------------------------------------------------- */
/* FluidSystem::FluidSystem (fluidsystem.cu:18-22): parameters take the
 * FluidParams constructor defaults (fluidparams.cuh:81-97).  device < 0 uses
 * the current CUDA device. */
int sph_create(sph_system** out, int device);
/* FluidSystem::~FluidSystem (fluidsystem.cu:27-31) */
int sph_destroy(sph_system* s);
/* FluidSystem::clear (fluidsystem.cu:36-52) */
int sph_clear(sph_system* s);
/* FluidSystem::init (fluidsystem.cu:196-265): unit cube, res^3 cells, h=1/res,
 * parameter resets of fluidsystem.cu:202-235, zeroed state. */
int sph_init(sph_system* s, uint32_t num_points, uint32_t res);
/* FluidSystem::setup (fluidsystem.cu:132-147): init + one block [0.1,0.9]^3 */
int sph_setup(sph_system* s, uint32_t num_points, uint32_t res);
/* FluidSystem::setupFromData (fluidsystem.cu:179-189): init + copy */
int sph_setup_from_data(sph_system* s, const float* pos, const float* vel, uint32_t n, uint32_t res);
/* FluidSystem::createFluidBlock (fluidsystem.cu:66-127), protected in the
 * reference and used by its subclasses (test/src/myfluidsystem.cpp:14-30). */
int sph_create_block(sph_system* s, uint32_t first, uint32_t n, float min_x, float min_y, float min_z,
                     float max_x, float max_y, float max_z);
/* Overwrite positions (and velocities when vel != NULL) of all particles;
 * accelerations are zeroed, as after init.  The copy half of setupFromData. */
int sph_set_state(sph_system* s, const float* pos, const float* vel, uint32_t n);

/* ---- stepping ---------------------------------------------------------- */
/* FluidSystem::advance (fluidsystem.cu:273-399).  Runs the substeps the
 * reference's float loop `for (dt = part; dt <= full; dt += part)` would run
 * (e.g. advance(0.01, 10) runs 9), each with dt = full_dt/substeps.  Blocks
 * until the work is done.  *executed (may be NULL) receives the count.
 * A loop that would never terminate in the reference returns SPH_EINVAL.
 * Without debug taps it then starts the next substep's sort and density
 * pass before returning, which the next advance or an export needs; errors
 * that pass raises are returned by the next call. */
int sph_advance(sph_system* s, float full_dt, uint32_t substeps, uint32_t* executed);
/* As sph_advance but returns after enqueueing; pair with sph_sync. */
int sph_advance_async(sph_system* s, float full_dt, uint32_t substeps, uint32_t* executed);
int sph_sync(sph_system* s);
/* Substep count of the reference loop, without running it. */
int64_t sph_substep_count(float full_dt, uint32_t substeps);

/* ---- readback ---------------------------------------------------------- */
/* FluidSystem::exportToData (fluidsystem.cu:154-173): positions, density
 * colour (DensityColourOperator, fluidutil.cu:67-80) and velocities in the
 * order of the last substep's cell sort.  Any pointer may be NULL.  Returns
 * once the buffers are filled; the next substep's force pass may then be
 * running already (sph_set_export_ahead). */
int sph_export(sph_system* s, float* pos, float* colour, float* vel, uint32_t n);
/* Houdini PGEOMETRY V5 export of one frame, byte-identical to fluidtest's
 * dumpToGeo (test/src/main.cpp:10-74): pos/colour/vel packed xyz, n points.
 * sph_geo_path formats "<filebase>.<frame:04d>.geo" (test/src/main.cpp:17-18). */
int sph_write_geo(const char* path, const float* pos, const float* colour, const float* vel, uint32_t n,
                  float pscale);
int sph_geo_path(char* out, uint64_t cap, const char* filebase, uint32_t frame);
/* FluidSystem::getPscale (fluidsystem.cu:406-409) */
int sph_get_pscale(const sph_system* s, float* out);
uint32_t sph_num_particles(const sph_system* s);
int sph_is_init(const sph_system* s);

/* ---- parameters: FluidSystem setters (fluidsystem.cu:412-475) ---------- */
int sph_set_rest_density(sph_system* s, float v);   /* setRestDensity */
int sph_set_particle_size(sph_system* s, float v);  /* setParticleSize */
int sph_set_gas_constant(sph_system* s, float v);   /* setGasConstant */
int sph_set_limits(sph_system* s, float vel_limit, float acc_limit); /* setLimits */
int sph_set_xsph_scale(sph_system* s, float v);     /* setXSPHScale */
int sph_set_surface_tension(sph_system* s, float v);/* setSurfaceTension */
int sph_set_viscosity(sph_system* s, float v);      /* setViscosity */
int sph_set_adhesion(sph_system* s, float v);       /* setAdhesion */
int sph_set_vdamp(sph_system* s, float v);          /* setVDamp */
int sph_set_gamma(sph_system* s, float v);          /* setGamma */
int sph_set_mass(sph_system* s, float v);           /* setMass */
/* Additions (no reference setter): gravity is fixed at (0,-9.8,0) in the
 * reference (fluidparams.cuh:97); the domain is the unit cube (fluidutil.cu:85-102). */
int sph_set_gravity(sph_system* s, float gx, float gy, float gz);
/* Rectangular box [0,lx]x[0,ly]x[0,lz] with cell size h (the smoothing
 * length).  Reallocates the grid; particle state is kept. */
int sph_set_domain(sph_system* s, float lx, float ly, float lz, float h);
/* Boundary shape.  The reference's boundarySDF (fluidutil.cu:85-102) returns
 * the box distance; it also computes, and discards, the distance to the
 * sphere of radius 0.5 about the cube's centre.  SPH_BOUNDARY_SPHERE uses
 * that sphere (radius: the box's smallest half extent, about its centre) for
 * the boundary density, adhesion and the integrator's boundary projection.
 * The grid still covers the box. */
#define SPH_BOUNDARY_BOX 0
#define SPH_BOUNDARY_SPHERE 1
int sph_set_boundary(sph_system* s, int shape);
int sph_get_boundary(const sph_system* s, int* shape);

/* Whole parameter set, for inspection and bulk configuration. */
typedef struct sph_params {
    uint32_t box_mode;   /* 0: unit cube with res cells per axis; 1: box lx,ly,lz with cell h */
    uint32_t res;
    float lx, ly, lz, h;
    float rest_density, gas_constant, gamma, mass, particle_size;
    float xsph, surface_tension, viscosity, adhesion, vdamp;
    float vel_limit, acc_limit, dt;
    float gravity[3];
} sph_params;
int sph_get_params(const sph_system* s, sph_params* out);
int sph_set_params(sph_system* s, const sph_params* p);

/* Derived device parameter block as doubles, in this order: gx, gy, gz,
 * inv_cell, h, h2, poly6, grad_poly6, grad_spiky, cohesion, invh9,
 * rest_density, gas_constant, gamma, mass, particle_size, dt, xsph,
 * surface_tension, viscosity, adhesion, vdamp, vel_limit, acc_limit,
 * gravity xyz, eps.  Returns the number written. */
int sph_get_derived(const sph_system* s, double* out, int cap);
/* The same derivation for a parameter set, without a device (host only). */
int sph_derive_params(const sph_params* p, double* out, int cap);

/* ---- snapshot / resume ---------------------------------------------------
 * No counterpart in the reference (it has no checkpointing).  A snapshot is
 * a 128-byte header (magic, version, particle count, the parameter set in
 * force) followed by positions, velocities and accelerations of every
 * particle as 4 floats each (xyz and the slot's w lane), in the current
 * slot order: sph_snapshot_bytes(n) = 128 + 48 n bytes, little endian.
 * Restoring into a system holding the same particle count (any parameters)
 * replaces its parameters and state; stepping then continues bit for bit as
 * the snapshotted system would have.  Errors: SPH_EINVAL for a short
 * buffer, a bad magic/version or a particle-count mismatch. */
#define SPH_SNAPSHOT_MAGIC 0x53485053u   /* "SPHS" */
#define SPH_SNAPSHOT_VERSION 1u
typedef struct sph_snapshot_header {
    uint32_t magic;
    uint32_t version;
    uint32_t n;
    uint32_t header_bytes;   /* 128 */
    sph_params params;
    uint32_t reserved[6];    /* [0]: boundary shape (SPH_BOUNDARY_*); others 0 */
} sph_snapshot_header;
uint64_t sph_snapshot_bytes(uint32_t n);
int sph_snapshot(sph_system* s, void* buf, uint64_t cap, uint64_t* written);
int sph_restore(sph_system* s, const void* buf, uint64_t bytes);

/* ---- parity / debug taps ----------------------------------------------- */
/* Per-particle and per-cell intermediates of the last substep, indexed like
 * the reference's device vectors after that substep (cell order). */
enum sph_field {
    SPH_FIELD_HASH = 0,       /* u32[n]  m_Hash after the sort (NULL_HASH = 0xFFFFFFFF) */
    SPH_FIELD_PERM = 1,       /* u32[n]  pre-sort index of the particle now at each slot */
    SPH_FIELD_CELLSTART = 2,  /* u32[cells] m_ScatterAddress */
    SPH_FIELD_CELLOCC = 3,    /* u32[cells] m_CellOcc */
    SPH_FIELD_NBRCOUNT = 4,   /* u32[n]  neighbours j != i with r^2 <= h^2 (needs debug taps) */
    SPH_FIELD_DENSITY = 5,    /* f32[n]  m_Density */
    SPH_FIELD_PRESSURE = 6,   /* f32[n]  m_Pressure */
    SPH_FIELD_SOUNDSPEED = 7, /* f32[n]  m_SoundSpeed */
    SPH_FIELD_FPRESSURE = 8,  /* f32[3n] pressure force (needs debug taps) */
    SPH_FIELD_FTENSION = 9,   /* f32[3n] tension force (needs debug taps) */
    SPH_FIELD_FADHESION = 10, /* f32[3n] adhesion force (needs debug taps) */
    SPH_FIELD_FVISCOSITY = 11,/* f32[3n] viscosity force (needs debug taps) */
    SPH_FIELD_NORMAL = 12,    /* f32[3n] m_Normals (surface tension scenes only) */
    SPH_FIELD_POS_SORTED = 13,/* f32[3n] positions in cell order before integration */
    SPH_FIELD_ACC = 14,       /* f32[3n] m_Acceleration */
    SPH_FIELD_VEL_INT = 15    /* f32[3n] velocity after integration, before XSPH */
};
/* Enable the optional taps (neighbour counts, force components).  With taps
 * on, every field describes the last substep run.  Without them, the sort
 * fields (hash, perm, cell start and occupancy) and density, pressure and
 * sound speed describe the most recent sort, which after a blocking advance
 * or an export is already the next substep's (its prefix runs early, see
 * sph_advance), and after an export the normals may be the next substep's
 * too (sph_set_export_ahead). */
int sph_debug_enable(sph_system* s, int on);
int sph_debug_get(sph_system* s, int field, void* buf, uint64_t count);
/* Test control of the error path of the cell scan (no counterpart: the
 * reference's scan is thrust's, which cannot fail this way).  The scan's
 * look-back waits give up after spin_limit polls (0: the default, 2^22)
 * and then report SPH_ETIMEOUT.  With withhold_first_tile != 0 no block of
 * the scan takes the first tile of cells, so every wait that reaches it
 * runs out: the step returns SPH_ETIMEOUT, no pass after the scan touches
 * the particles, and the state stays as it was before the failed substep.
 * sph_debug_scan_fault(s, 0, 0) restores normal operation. */
int sph_debug_scan_fault(sph_system* s, uint32_t spin_limit, int withhold_first_tile);

/* ---- execution options and profiling ----------------------------------- */
/* How the substep is launched (no effect on results: every choice computes
 * the same values bit for bit).  tile: particles per tile = threads per
 * block (64, 128 or 256); persistent: 0 = one block per tile, k > 0 = k
 * blocks per SM taking tiles from a counter in the neighbour passes; skin:
 * neighbour-mask skin in units of h, in (0, 1]; variant: SPH_VARIANT_* bits
 * choosing how the neighbour walks are scheduled.  Defaults: tile 128,
 * persistent 0, skin 0.1, variant 63 (per-row density and XSPH walks,
 * 64-register force build; force and normal passes walk a row table; the
 * density scan split over three threads per particle in launches of at most
 * 49,152 particles). */
#define SPH_VARIANT_DENSITY_ROWS   0x1u  /* density: one loop per cell row */
#define SPH_VARIANT_XSPH_ROWS      0x2u  /* XSPH: one loop per cell row */
#define SPH_VARIANT_FORCE_OCC      0x4u  /* force: 64-register build, more resident warps */
#define SPH_VARIANT_FORCE_TABLE    0x8u  /* force: row table in shared memory */
#define SPH_VARIANT_NORMALS_TABLE  0x10u /* normals: row table in shared memory */
#define SPH_VARIANT_DENSITY_SPLIT  0x20u /* density: three threads per particle share the candidate
                                            scan (with DENSITY_ROWS, one block per tile, no skin
                                            words; launches of at most 49,152 particles) */
typedef struct sph_exec_config {
    uint32_t tile;
    uint32_t persistent;
    float skin;
    uint32_t variant;
} sph_exec_config;
int sph_set_exec(sph_system* s, const sph_exec_config* e);
/* XSPH schedule (no counterpart: the reference ends every substep with its
 * XSPH pass).  on != 0, the default: a substep ends after the integrator and
 * its XSPH update is applied by the next substep's density pass, in the same
 * neighbour walk; reading a system's state (export, snapshot) computes the
 * update on demand without changing the run.  The pairs are exactly the
 * reference's (its previous cell lists are honoured); only the summation
 * order of the XSPH sums differs from the per-substep schedule (on == 0).
 * Debug taps imply the per-substep schedule, as do grids of more than 1024
 * cells along an axis. */
int sph_set_deferred_xsph(sph_system* s, int on);
int sph_get_exec(const sph_system* s, sph_exec_config* e);
int sph_set_use_graph(sph_system* s, int on);     /* CUDA-graph replay of the substep (default on) */
/* Export ahead (no counterpart; on != 0 is the default).  An export of
 * velocities after a blocking advance waits for the next substep's density
 * pass, which computes the XSPH update.  With this on, that export also
 * starts the next substep's normal and force passes while the velocities
 * cross the host link.  The next advance takes them as its first substep
 * when no parameter changed; every other call first undoes them exactly.
 * Results are the same bit for bit either way. */
int sph_set_export_ahead(sph_system* s, int on);
/* out[0]: exports that ran passes ahead; out[1]: of those, taken by an
 * advance; out[2]: undone (out[0] = out[1] + out[2], plus one while passes
 * wait to be taken).  After two undone in a row the next 16 exports run
 * nothing ahead. */
int sph_export_ahead_stats(const sph_system* s, uint64_t* out);
int sph_set_profiling(sph_system* s, int on);     /* per-pass CUDA events (disables the graph) */
/* Accumulated per-pass milliseconds since profiling was enabled, in the
 * order hash, scan, sort, density, normals, force_integrate, xsph, substep. */
int sph_get_pass_times(sph_system* s, double* ms, int cap, uint64_t* substeps);
const char* sph_pass_name(int i);
/* Page-lock (or release) a caller's host buffer so transfers to and from
 * it run at full link speed (cudaHostRegister). */
int sph_host_register(void* ptr, uint64_t bytes);
int sph_host_unregister(void* ptr);
/* Device timing on the handle's stream: record CUDA event `slot` (0..63);
 * elapsed milliseconds between two recorded slots (waits for slot b). */
int sph_timer_mark(sph_system* s, int slot);
int sph_timer_elapsed(sph_system* s, int a, int b, float* ms);
const char* sph_last_error(const sph_system* s);
const char* sph_version(void);

/* ---- batched step -------------------------------------------------------
 * Many independent scenes (each a FluidSystem with its own domain, parameters
 * and particle count) advanced together: every pass of the substep is one
 * launch over all live scenes (segmented hash and sort with per-scene cell
 * ranges, scene-aware neighbour kernels), and the whole substep is replayed
 * as one CUDA graph.  No counterpart in the reference, which holds one
 * parameter block per process (fluidparams.cu:6) and so one system at a time. */
typedef struct sph_batch sph_batch;
typedef struct sph_lattice {
    float lo[3];            /* block corner */
    float spacing;          /* lattice spacing */
    uint32_t nx, ny, nz;    /* sites per axis; particle (ix*ny+iy)*nz+iz */
    float jitter;           /* uniform jitter amplitude (+/-), seeded */
    float vel[3];           /* initial velocity */
    uint32_t pad_;
    uint64_t seed;
} sph_lattice;
int sph_batch_create(sph_batch** out, int device);
int sph_batch_destroy(sph_batch* b);
/* Add a scene of n particles with parameters p (p->dt is its substep dt);
 * state starts at zero.  Returns its id in *scene_id. */
int sph_batch_add_scene(sph_batch* b, const sph_params* p, uint32_t n, int* scene_id);
int sph_batch_remove_scene(sph_batch* b, int scene_id);
int sph_batch_set_params(sph_batch* b, int scene_id, const sph_params* p);
int sph_batch_set_state(sph_batch* b, int scene_id, const float* pos, const float* vel, uint32_t n);
/* Fill particles [first, first + nx*ny*nz) of a scene with a jittered
 * lattice block generated on the device. */
int sph_batch_generate_lattice(sph_batch* b, int scene_id, const sph_lattice* spec, uint32_t first);
/* Advance every live scene by `substeps` substeps of its own dt (blocking).
 * substeps == 0 only prepares the next step (scene layout, parameters and
 * CUDA graphs after scenes joined or left) and launches nothing. */
int sph_batch_step(sph_batch* b, uint32_t substeps);
int sph_batch_step_async(sph_batch* b, uint32_t substeps);
int sph_batch_sync(sph_batch* b);
int sph_batch_get_state(sph_batch* b, int scene_id, float* pos, float* colour, float* vel, uint32_t n);
int sph_batch_set_boundary(sph_batch* b, int scene_id, int shape);
/* Snapshot / resume of one scene, in the sph_snapshot format (above). */
int sph_batch_snapshot(sph_batch* b, int scene_id, void* buf, uint64_t cap, uint64_t* written);
int sph_batch_restore(sph_batch* b, int scene_id, const void* buf, uint64_t bytes);
uint32_t sph_batch_num_scenes(const sph_batch* b);
uint64_t sph_batch_num_particles(const sph_batch* b);
int sph_batch_debug_enable(sph_batch* b, int on);
int sph_batch_debug_get(sph_batch* b, int scene_id, int field, void* buf, uint64_t count);
int sph_batch_set_use_graph(sph_batch* b, int on);
int sph_batch_set_exec(sph_batch* b, const sph_exec_config* e);
int sph_batch_set_deferred_xsph(sph_batch* b, int on);
int sph_batch_timer_mark(sph_batch* b, int slot);
int sph_batch_timer_elapsed(sph_batch* b, int a, int b2, float* ms);
/* Per-pass CUDA-event timing of the batch's substeps, as sph_set_profiling /
 * sph_get_pass_times: one launch per pass covers every scene. */
int sph_batch_set_profiling(sph_batch* b, int on);
int sph_batch_get_pass_times(sph_batch* b, double* ms, int cap, uint64_t* substeps);
const char* sph_batch_last_error(const sph_batch* b);

/* ---- served step (continuous batching) ----------------------------------
 * A request loop on its own host thread.  Requests (a scene: parameters,
 * initial state, number of substeps) are queued as they arrive and admitted
 * in arrival order while the device-memory budget and the live-scene limit
 * allow; admitted scenes stay resident on the GPU and every loop iteration
 * advances all live scenes by one substep in one batched step; a scene that
 * has run its substeps is copied to the host and leaves, freeing memory for
 * the queue.  No counterpart in the reference. */
typedef struct sph_server sph_server;
typedef struct sph_server_config {
    int device;                 /* CUDA device, -1 = current */
    uint64_t memory_budget;     /* device bytes the scenes may occupy */
    uint32_t max_live_scenes;   /* 0 = no limit */
    uint32_t substeps_per_iteration; /* substeps between admissions (>= 1) */
} sph_server_config;
typedef struct sph_request {
    sph_params params;          /* domain and physics; params.dt is the substep */
    uint32_t n;                 /* particles */
    uint32_t steps;             /* substeps to run */
    const float* pos;           /* initial positions (host, packed xyz), or NULL to use blocks */
    const float* vel;           /* initial velocities, or NULL for zero */
    const sph_lattice* blocks;  /* lattice blocks generated on the device (when pos == NULL) */
    uint32_t num_blocks;
    uint32_t pad_;
} sph_request;
enum sph_request_state { SPH_REQ_QUEUED = 0, SPH_REQ_RUNNING = 1, SPH_REQ_DONE = 2, SPH_REQ_FAILED = 3,
                         SPH_REQ_UNKNOWN = 4 };
typedef struct sph_server_stats {
    uint64_t submitted, admitted, completed, failed, rejected;
    uint64_t iterations;        /* batched steps run */
    uint64_t particle_steps;    /* sum over completed and live scenes */
    double busy_seconds;        /* time spent stepping */
    uint32_t live_scenes, queued;
    uint64_t live_particles;
    uint64_t device_bytes;      /* arena footprint */
    uint64_t peak_live_particles;
    double admit_seconds;       /* creating admitted scenes (initial state upload or lattice) */
    double read_seconds;        /* reading finished scenes back and removing them */
    double layout_seconds;      /* host work of membership changes (tile tables, parameters), part of busy */
    uint64_t admit_retries;     /* admissions put back because the arena had no room yet */
} sph_server_stats;
int sph_server_create(sph_server** out, const sph_server_config* cfg);
/* Stops the loop (running scenes are abandoned) and frees everything. */
int sph_server_destroy(sph_server* s);
/* Queue a request; the input arrays are copied.  SPH_EBUSY if it can never
 * fit the memory budget. */
int sph_server_submit(sph_server* s, const sph_request* req, uint64_t* request_id);
int sph_server_state(sph_server* s, uint64_t request_id);
/* Wait until the request is done or failed, at most timeout_ms (< 0: no
 * limit); SPH_ETIMEOUT if it is still pending. */
int sph_server_wait(sph_server* s, uint64_t request_id, int64_t timeout_ms);
/* Copy a finished request's final positions and velocities (either may be
 * NULL) and release it. */
int sph_server_fetch(sph_server* s, uint64_t request_id, float* pos, float* vel, uint32_t n);
/* Seconds since server start at submission, admission and completion. */
int sph_server_times(sph_server* s, uint64_t request_id, double* t_submit, double* t_admit, double* t_done);
int sph_server_get_stats(sph_server* s, sph_server_stats* out);
/* Block until the queue is empty and no scene is live (or timeout). */
int sph_server_drain(sph_server* s, int64_t timeout_ms);
const char* sph_server_last_error(sph_server* s);

/* ---- allocation-free cell-start scan ------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (an application that owns all device memory through its own arena, or a
 * frame loop where an allocation would stall the device): exclusive scan of
 * n per-cell particle counts (device u32[n]) into cell starts (device
 * u32[n+1], starts[n] = total), the step fluidsystem.cu:316 performs, with
 * its scratch in a fixed 128 KiB array inside the library instead of a
 * cudaMalloc.  n must be 1..SPH_NOALLOC_MAX_CELLS, else SPH_EINVAL.
 * Enqueued on `stream` (a cudaStream_t; NULL = legacy default stream) on
 * the current device; it does not synchronise.  Each call looks up the
 * scratch address in the current context (cudaGetSymbolAddress), so the call
 * stays valid after the application resets the device; the first call on a
 * device may also load the library's device code (lazy module loading), so
 * make that first call before any stream capture.  Every call shares the
 * scratch: calls that overlap on the GPU race and must be serialised by the
 * caller. */
#define SPH_NOALLOC_MAX_TILES 32768u
#define SPH_NOALLOC_MAX_CELLS (SPH_NOALLOC_MAX_TILES * 4096u)
int sph_scan_cells_noalloc(const uint32_t* counts, uint32_t n, uint32_t* starts, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SPH_C_H */
