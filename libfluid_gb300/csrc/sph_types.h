// Plain-old-data types shared by host code and sm_103a kernels.
//
// One scene = one independent fluid system (a FluidSystem in the reference,
// libfluid/include/fluidsystem.h:16-126).  The reference keeps one parameter
// block per process in __constant__ memory (fluidparams.cu:6); here every
// scene has its own DevParams in global memory so that many scenes can be
// advanced by one launch per pass.
#pragma once
#include <stdint.h>

#define SPH_NULL_HASH 0xFFFFFFFFu   // fluiddefines.h:12 (UINT_MAX)
#define SPH_OKEY_NULL 0xFFFFFFFFu   // packed cell of a particle outside the grid
#define SPH_OKEY_MOVED 0x80000000u  // packed-cell flag: the particle has changed cell since
#define SPH_OKEY_MAX_DIM 1024u      // grids up to this many cells per axis can defer XSPH
#define SPH_FLAG_DEFER_XSPH 0x2u    // DevParams.flags: XSPH applied by the next density pass
#define SPH_FLAG_SPHERE 0x4u        // DevParams.flags: sphere boundary instead of the box

// Derived per-scene parameters (the FluidParamData of fluidparams.cuh:16-69,
// generalised to a rectangular box [0,L]^3 with cell size h).
struct DevParams {
    // grid: cell = floor(p * inv_cell) per axis, linearised x fastest
    uint32_t gx, gy, gz, gxy;     // grid dims and gx*gy
    uint32_t ncells;              // gx*gy*gz; the scene's NULL bucket is cell ncells
    float inv_cell;               // float(res) for the unit cube
    // box signed distance: d = |p - c| - b (fluidutil.cu:85-102)
    float box_cx, box_cy, box_cz, box_bx, box_by, box_bz;
    // smoothing length and kernel constants (fluidparams.cu:51-89)
    float h, halfh, h2, h4, h6, h8, h9, invh9;
    float poly6, grad_poly6, grad_spiky, cohesion;
    float visc_eps;               // 0.01*h^2 (fluidphysics.cu:279), rounded to float once
    // fluid
    float rest_density, inv_rest_density, gas_constant, gamma, eos_k;  // eos_k = B*rho0/gamma
    float mass, two_mass, particle_size, inv_particle_size;
    float dt, dtdt;
    float xsph, surface_tension, viscosity, adhesion, vdamp;
    float vel_limit, acc_limit, vel_limit2, acc_limit2;
    float grav_x, grav_y, grav_z;
    float eps;                    // FLT_MIN (fluidparams.cu:48)
    uint32_t flags;               // bit0: surface tension active (normals pass needed);
                                  // bit1: the scene defers XSPH (SPH_FLAG_DEFER_XSPH);
                                  // bit2: sphere boundary (SPH_FLAG_SPHERE)
    float skin2;                  // ((1 + skin) h)^2: radius of the neighbour masks
    float inv_h2;                 // 1/h^2, normalises displacements for the XSPH mask check
    float xsph_disp_limit2;       // (skin/2)^2 * 0.98: largest (displacement/h)^2 XSPH may accept
    float sphere_r;               // sphere boundary (flags bit2): radius about the box centre
    uint32_t pad_[2];
};

// Neighbour masks are built with radius (1 + skin) h (default skin below).
// XSPH, which runs on positions moved by the integrator, may use them only
// while every particle moved less than skin*h/2 in the substep (checked on
// the device; otherwise XSPH walks all candidates).
#define SPH_SKIN_DEFAULT 0.1f

// Neighbour-mask rows per slot (row m of slot k at mask[m * stride + k]).
// Exact-neighbour words of a cell row: rows of up to 64 candidates carry two
// words (word h: candidates jb + 32h .. jb + 32h + 31; the second is written
// and read only for rows longer than 32); longer rows carry none and are
// walked in full.  Words of row r sit at mask rows SPH_MASK_EXACT + 2r + h.
#define SPH_MASK_SKIN   0u    // 9 rows: candidates within the skin radius (rows of <= 32)
#define SPH_MASK_EXACT  9u    // 18 rows: neighbours r^2 <= h^2, j != i (readers test r^2 > eps)
#define SPH_MASK_ROWS   27u
#define SPH_WIDE_ROW    64u   // longest row with mask words
#define SPH_ROW_TABLE_WORDS 27u   // per-thread row table: 9 row starts + 18 words

// Kernel variants (bits of the execution config's `variant`). All variants
// visit neighbours in the same order and give identical results; they differ
// only in how the walk is scheduled.
#define SPH_VARIANT_DENSITY_ROWS  0x1u   // density: one loop per cell row, four candidates in flight (two 256-bit loads)
#define SPH_VARIANT_XSPH_ROWS     0x2u   // XSPH: one loop per cell row instead of one flattened walk
#define SPH_VARIANT_FORCE_OCC     0x4u   // force: 64-register build (more resident warps)
#define SPH_VARIANT_FORCE_TABLE   0x8u   // force: walk over a per-thread row table in shared memory
#define SPH_VARIANT_NORMALS_TABLE 0x10u  // normals: the same
#define SPH_VARIANT_DENSITY_SPLIT 0x20u  // density: three threads per particle share the candidate scan
                                         // (launches of at most SPH_DENSITY_SPLIT_MAX particles)
#define SPH_VARIANT_MASK          0x3fu
#define SPH_VARIANT_DEFAULT       0x3fu  // measured fastest on the 1M dam break, the 256-scene batch
                                         // and the 8M tension scene (where the split scan does not
                                         // apply), and on dam breaks of 8,000 to 32,768 particles
// Largest launch (particles over all tiles) that the split scan serves: it
// gained 6-9% per substep on dam breaks of 8,000 to 32,768 particles and lost
// 10% at 64,000 (the blocks of three times the threads run fewer at once).
#ifndef SPH_DENSITY_SPLIT_MAX
#define SPH_DENSITY_SPLIT_MAX     49152u
#endif

// Scene placement in the engine's arenas.
struct DevScene {
    uint32_t part_base;   // first particle slot of the scene
    uint32_t n;           // particle count
    uint32_t cell_base;   // first cell of the scene in the packed cell arena
    uint32_t ncells;      // real cells; the NULL bucket follows at cell_base+ncells
};

// A tile: up to SPH_TILE consecutive particle slots of one scene.
// x = scene, y = first slot, z = count, w = 0.
#define SPH_TILE 256

// Status bits raised by kernels (read back after a step).
#define SPH_STATUS_CELL_OVERFLOW 0x1u   // a cell held more particles than the rank pass supports
#define SPH_STATUS_NONFINITE     0x2u   // a non-finite position appeared
#define SPH_STATUS_SCAN_TIMEOUT  0x4u   // a wait of the cell scan's look-back ran out

// Maximum particles one cell (or a scene's NULL bucket) may hold.  The
// reference cannot launch more than 1024 threads per cell block
// (fluidsystem.cu:322); this build supports 8x that.
#define SPH_MAX_CELL_OCC 8192u

// Lattice block generator (a dam-break fluid block with seeded jitter).
struct LatticeSpec {
    float lo[3];          // block corner
    float spacing;        // lattice spacing
    uint32_t nx, ny, nz;  // lattice sites per axis (x outermost, z innermost)
    float jitter;         // uniform jitter amplitude (+/-)
    float vel[3];         // initial velocity
    uint32_t pad_;
    uint64_t seed;
};
