// Device-side building blocks of the WCSPH step: box SDF, smoothing kernels,
// spatial hash.  The library is compiled with -fmad=false: every fused
// multiply-add below is written out with fmaf() so that the arithmetic is
// fixed and identical to the CPU oracle's.  The fused points are:
//   dot(a,b)        = fma(a.z,b.z, fma(a.y,b.y, a.x*b.x))
//   h2 - r*r        = fma(-r, r, h2)
//   running sums    = fma(a, b, s)
// The reference build lets nvcc choose (it contracts by default); results
// differ from it by a few ulp, within the tolerances of the parity tests.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "sph_types.h"

namespace sph {

// helper_math's dot, a.x*b.x + a.y*b.y + a.z*b.z, as the reference build
// evaluates it: nvcc fuses the x product into the first add and the z
// product into the second.  The order decides r^2 to the last bit, and with
// it whether a pair at r = h counts and how large (h - r) is.
__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return fmaf(az, bz, fmaf(ax, bx, ay * by));
}

// Box signed distance, negative inside (boundarySDF, fluidutil.cu:85-102).
__device__ __forceinline__ float sdf_box(const DevParams& P, float x, float y, float z) {
    const float qx = fabsf(x - P.box_cx) - P.box_bx;
    const float qy = fabsf(y - P.box_cy) - P.box_by;
    const float qz = fabsf(z - P.box_cz) - P.box_bz;
    const float inner = fminf(fmaxf(qx, fmaxf(qy, qz)), 0.0f);
    const float px = fmaxf(qx, 0.0f), py = fmaxf(qy, 0.0f), pz = fmaxf(qz, 0.0f);
    return inner + sqrtf(dot3(px, py, pz, px, py, pz));
}

// Sphere container: length(p - c) - r (the distance boundarySDF computes but
// does not return, fluidutil.cu:97-98), c the box centre, r its smallest half
// extent (0.5 in the unit cube, as there).
__device__ __forceinline__ float sdf_sphere(const DevParams& P, float x, float y, float z) {
    const float dx = x - P.box_cx, dy = y - P.box_cy, dz = z - P.box_cz;
    return sqrtf(dot3(dx, dy, dz, dx, dy, dz)) - P.sphere_r;
}
// The scene's boundary distance, negative inside.
__device__ __forceinline__ float sdf(const DevParams& P, float x, float y, float z) {
    return (P.flags & SPH_FLAG_SPHERE) ? sdf_sphere(P, x, y, z) : sdf_box(P, x, y, z);
}

// Central-difference SDF normal (boundaryNormalSDF, fluidutil.cu:104-112),
// normalised as v * (1/sqrt(v.v)).
__device__ __forceinline__ float3 sdf_normal(const DevParams& P, float x, float y, float z) {
    const float e = 0.0001f;
    const float nx = sdf(P, x + e, y, z) - sdf(P, x - e, y, z);
    const float ny = sdf(P, x, y + e, z) - sdf(P, x, y - e, z);
    const float nz = sdf(P, x, y, z + e) - sdf(P, x, y, z - e);
    const float inv = 1.0f / sqrtf(dot3(nx, ny, nz, nx, ny, nz));
    return make_float3(nx * inv, ny * inv, nz * inv);
}

// poly6 (fluidkernel.cu:5-8); the cube is formed by multiplication.
__device__ __forceinline__ float poly6(const DevParams& P, float r) {
    const float x = fmaf(-r, r, P.h2);
    return (r >= P.h) ? 0.0f : P.poly6 * (x * x * x);
}
// grad poly6 (fluidkernel.cu:10-13)
__device__ __forceinline__ float grad_poly6(const DevParams& P, float r) {
    const float x = fmaf(-r, r, P.h2);
    return (r >= P.h) ? 0.0f : P.grad_poly6 * r * (x * x);
}
// grad spiky (fluidkernel.cu:25-28)
__device__ __forceinline__ float grad_spiky(const DevParams& P, float r) {
    return (r >= P.h) ? 0.0f : P.grad_spiky * (P.h - r) * (P.h - r);
}
// cohesion (fluidkernel.cu:35-38) with the reference's operator precedence:
// the coefficient times (r > h/2) only selects the branch.
__device__ __forceinline__ float cohesion_k(const DevParams& P, float r) {
    if (r >= P.h) return 0.0f;
    const float sel = P.cohesion * (r > P.halfh ? 1.0f : 0.0f);
    const float hr = P.h - r;
    const float hr3 = hr * hr * hr;
    if (sel != 0.0f) return hr3 * r * r * r;
    return 2.0f * hr3 * r * r * r - P.h6 * 0.0156f;
}
// boundaryDensity (fluidkernel.cu:45-67), multiply-adds fused as the
// reference build fuses them (see the oracle).
__device__ __forceinline__ float boundary_density(const DevParams& P, float d) {
    if ((d > P.h) || (d < 0.0f)) return 0.0f;
    const float c = -d, c2 = c * c, c3 = c2 * c, c4 = c3 * c, c6 = c3 * c3;
    const float e1 = fmaf(35.0f, c6, -((180.0f * c4) * P.h2));
    const float e2 = fmaf(378.0f * c2, P.h4, e1);
    const float e3 = fmaf(-420.0f, P.h6, e2);
    const float poly = fmaf(c3, e3, (315.0f * c) * P.h8) + 128.0f * P.h9;
    return 1.0f - (0.0039062f * P.invh9) * poly;
}

// Grid coordinates of a position: floor(p * inv_cell) converted with
// round-toward-zero saturation (grid_from_point, fluidutil.cu:15-18).
__device__ __forceinline__ int3 grid_of(const DevParams& P, float x, float y, float z) {
    return make_int3(__float2int_rz(floorf(x * P.inv_cell)), __float2int_rz(floorf(y * P.inv_cell)),
                     __float2int_rz(floorf(z * P.inv_cell)));
}
__device__ __forceinline__ bool grid_inside(const DevParams& P, int3 g) {
    return g.x >= 0 && g.x < (int)P.gx && g.y >= 0 && g.y < (int)P.gy && g.z >= 0 && g.z < (int)P.gz;
}
// Scene-local cell index, or P.ncells (the scene's NULL bucket) outside the
// grid (cell_from_grid, fluidutil.cu:29-39, NULL_HASH -> bucket ncells).
__device__ __forceinline__ uint32_t cell_of(const DevParams& P, float x, float y, float z) {
    const int3 g = grid_of(P, x, y, z);
    return grid_inside(P, g) ? (uint32_t)g.x + (uint32_t)g.y * P.gx + (uint32_t)g.z * P.gxy : P.ncells;
}

// A particle's cell packed as x | y << 10 | z << 20 (grids of at most 1024
// cells per axis; larger grids run XSPH every substep), or SPH_OKEY_NULL
// outside the grid.  Kept from one substep to the next for deferred XSPH.
__device__ __forceinline__ uint32_t pack_cell(int3 g) {
    return (uint32_t)g.x | ((uint32_t)g.y << 10) | ((uint32_t)g.z << 20);
}
// Both packed cells exist and differ by at most one in every axis (one is in
// the other's 27-cell neighbourhood).  Bit 31 (SPH_OKEY_MOVED) is ignored.
__device__ __forceinline__ bool cells_adjacent(uint32_t a, uint32_t b) {
    if (b == SPH_OKEY_NULL) return false;
    const int dx = (int)(a & 1023u) - (int)(b & 1023u);
    const int dy = (int)((a >> 10) & 1023u) - (int)((b >> 10) & 1023u);
    const int dz = (int)((a >> 20) & 1023u) - (int)((b >> 20) & 1023u);
    return (unsigned)(dx + 1) <= 2u && (unsigned)(dy + 1) <= 2u && (unsigned)(dz + 1) <= 2u;
}
// The same for a pair already known to lie in each other's current 27-cell
// neighbourhood: when neither particle changed cell (no SPH_OKEY_MOVED bit,
// set by the hash pass), the previous cells are the current ones.
__device__ __forceinline__ bool cells_adjacent_fast(uint32_t a, uint32_t b) {
    return ((a | b) & SPH_OKEY_MOVED) == 0u || cells_adjacent(a, b);
}

// Visit the candidate neighbours of a particle in grid cell g: the 27 cells
// around it, clipped at the grid edge (fluidphysics.cu:30-34).  Cells
// (x-1..x+1, y, z) are consecutive in the x-fastest order and particles are
// sorted by cell, so each (y,z) row is one contiguous slot range.
// start[] is the exclusive scan of cell counts over the packed cell arena;
// delta maps it to particle slots.
template <class F>
__device__ __forceinline__ void for_candidates(const DevParams& P, const uint32_t* __restrict__ start,
                                               uint32_t cell_base, uint32_t delta, int3 g, F&& f) {
    const int x0 = max(g.x - 1, 0), x1 = min(g.x + 1, (int)P.gx - 1);
    const int z0 = max(g.z - 1, 0), z1 = min(g.z + 1, (int)P.gz - 1);
    const int y0 = max(g.y - 1, 0), y1 = min(g.y + 1, (int)P.gy - 1);
    for (int z = z0; z <= z1; ++z) {
        for (int y = y0; y <= y1; ++y) {
            const uint32_t row = cell_base + (uint32_t)y * P.gx + (uint32_t)z * P.gxy;
            const uint32_t jb = __ldg(start + row + x0) + delta;
            const uint32_t je = __ldg(start + row + x1 + 1) + delta;
            for (uint32_t j = jb; j < je; ++j) f(j);
        }
    }
}

// Row r (0..8) of the neighbourhood of grid cell g, dz = r/3-1, dy = r%3-1:
// the slot range [jb, je) of cells (x-1..x+1, y+dy, z+dz) clipped at the
// grid edge.  Returns false when the row lies outside the grid.  The rows are
// visited in the same order by every pass, so a candidate's (row, offset)
// names the same particle in the density, normal, force and XSPH passes.
__device__ __forceinline__ bool row_range(const DevParams& P, const uint32_t* __restrict__ start, uint32_t cell_base,
                                          uint32_t delta, int3 g, int r, uint32_t& jb, uint32_t& je) {
    const int z = g.z + r / 3 - 1, y = g.y + r % 3 - 1;
    if (z < 0 || z >= (int)P.gz || y < 0 || y >= (int)P.gy) return false;
    const int x0 = max(g.x - 1, 0), x1 = min(g.x + 1, (int)P.gx - 1);
    const uint32_t row = cell_base + (uint32_t)y * P.gx + (uint32_t)z * P.gxy;
    jb = __ldg(start + row + x0) + delta;
    je = __ldg(start + row + x1 + 1) + delta;
    return true;
}

// Visit the candidates recorded in a particle's neighbour masks: one 32-bit
// word per row, bit b = candidate jb+b lies within the skin radius
// (1 + SPH_SKIN) h at the positions the masks were built from.  Rows longer
// than 32 candidates carry no mask and are walked in full.  f(j) must apply
// its own exact distance test.
template <class F>
__device__ __forceinline__ void for_masked(const DevParams& P, const uint32_t* __restrict__ start, uint32_t cell_base,
                                           uint32_t delta, int3 g, const uint32_t* __restrict__ mask, size_t stride,
                                           uint32_t k, F&& f) {
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        uint32_t jb, je;
        if (!row_range(P, start, cell_base, delta, g, r, jb, je)) continue;
        if (je - jb <= 32u) {
            uint32_t bits = __ldg(mask + (size_t)r * stride + k);
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1u;
                f(jb + (uint32_t)b);
            }
        } else {
            for (uint32_t j = jb; j < je; ++j) f(j);
        }
    }
}

// Candidate walk over a particle's skin words, flattened across the 9
// rows: next() yields the next recorded candidate, moving to the next row
// inside the same call, so lanes of a warp never wait for each other at row
// boundaries.  Rows longer than 32 candidates carry no mask and yield every
// candidate (the caller's exact test decides).
struct MaskWalk {
    const DevParams& P;
    const uint32_t* __restrict__ start;
    uint32_t cell_base, delta;
    int3 g;
    const uint32_t* __restrict__ mask;
    size_t stride;
    uint32_t k;
    int r;
    uint32_t jb, je, j, bits;
    bool full;
    __device__ __forceinline__ MaskWalk(const DevParams& P_, const uint32_t* __restrict__ start_, uint32_t cb,
                                        uint32_t delta_, int3 g_, const uint32_t* __restrict__ mask_, size_t stride_,
                                        uint32_t k_)
        : P(P_), start(start_), cell_base(cb), delta(delta_), g(g_), mask(mask_), stride(stride_), k(k_), r(-1),
          jb(0), je(0), j(0), bits(0), full(false) {}
    __device__ __forceinline__ bool next(uint32_t& cand) {
        for (;;) {
            if (full) {
                if (j < je) { cand = j++; return true; }
                full = false;
            } else if (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1u;
                cand = jb + (uint32_t)b;
                return true;
            }
            if (++r >= 9) return false;
            if (!row_range(P, start, cell_base, delta, g, r, jb, je)) continue;
            if (je - jb <= 32u) bits = __ldg(mask + (size_t)r * stride + k);
            else { full = true; j = jb; }
        }
    }
};

// Walk of the exact-neighbour words of a particle's rows, flattened across
// the 9 rows and their halves.
struct WideMaskWalk {
    const DevParams& P;
    const uint32_t* __restrict__ start;
    uint32_t cell_base, delta;
    int3 g;
    const uint32_t* __restrict__ mask;   // exact rows (SPH_MASK_EXACT)
    size_t stride;
    uint32_t k;
    int r;
    uint32_t jb, je, j, bits, len;
    bool full, second;
    __device__ __forceinline__ WideMaskWalk(const DevParams& P_, const uint32_t* __restrict__ start_, uint32_t cb,
                                            uint32_t delta_, int3 g_, const uint32_t* __restrict__ mask_,
                                            size_t stride_, uint32_t k_)
        : P(P_), start(start_), cell_base(cb), delta(delta_), g(g_), mask(mask_), stride(stride_), k(k_), r(-1),
          jb(0), je(0), j(0), bits(0), len(0), full(false), second(false) {}
    __device__ __forceinline__ bool next(uint32_t& cand) {
        for (;;) {
            if (full) {
                if (j < je) { cand = j++; return true; }
                full = false;
            } else if (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1u;
                cand = jb + (uint32_t)b;
                return true;
            }
            if (!second && r >= 0 && len > 32u && len <= SPH_WIDE_ROW) {
                second = true;
                jb += 32u;
                bits = __ldg(mask + (size_t)(2 * r + 1) * stride + k);
                continue;
            }
            if (++r >= 9) return false;
            second = false;
            if (!row_range(P, start, cell_base, delta, g, r, jb, je)) { len = 0; continue; }
            len = je - jb;
            if (len > SPH_WIDE_ROW) { full = true; j = jb; }
            else bits = __ldg(mask + (size_t)(2 * r) * stride + k);
        }
    }
};

// Row table of one particle's neighbourhood, kept in the block's shared
// memory (a column per thread: entry e of thread t at tab[e*ts + t]):
// entries 0-8 the first slot jb of each row, 9-26 the rows' exact-neighbour
// words (entry 9 + 2r + h), or, for a row longer than 64 candidates, its
// length in entry 9 + 2r.  `live` has a bit per half-row (2r + h) with
// something to visit, `full` one (2r) per row walked in full.  The row
// starts and first words are loaded together; second words only for rows
// longer than 32.  TableWalk below moves between rows with two
// shared-memory reads instead of dependent global loads.
__device__ __forceinline__ void build_row_table(const DevParams& P, const uint32_t* __restrict__ start,
                                                uint32_t cell_base, uint32_t delta, int3 g,
                                                const uint32_t* __restrict__ mask, size_t stride, uint32_t k,
                                                uint32_t* tab, uint32_t ts, uint32_t& live, uint32_t& full) {
    live = 0u;
    full = 0u;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        uint32_t jb, je;
        const uint32_t w0 = __ldg(mask + (size_t)(2 * r) * stride + k);
        if (!row_range(P, start, cell_base, delta, g, r, jb, je)) continue;
        const uint32_t len = je - jb;
        tab[r * ts] = jb;
        if (len > SPH_WIDE_ROW) {
            full |= 1u << (2 * r);
            live |= 1u << (2 * r);
            tab[(9 + 2 * r) * ts] = len;
        } else {
            const uint32_t w1 = (len > 32u) ? __ldg(mask + (size_t)(2 * r + 1) * stride + k) : 0u;
            tab[(9 + 2 * r) * ts] = w0;
            tab[(10 + 2 * r) * ts] = w1;
            if (w0) live |= 1u << (2 * r);
            if (w1) live |= 1u << (2 * r + 1);
        }
    }
}

// Walk of a row table in WideMaskWalk's order (rows ascending, candidates of
// a row ascending).
struct TableWalk {
    const uint32_t* tab;
    uint32_t ts, live, full, jb, bits, j, je;
    __device__ __forceinline__ TableWalk(const uint32_t* tab_, uint32_t ts_, uint32_t live_, uint32_t full_)
        : tab(tab_), ts(ts_), live(live_), full(full_), jb(0), bits(0), j(0), je(0) {}
    __device__ __forceinline__ bool next(uint32_t& cand) {
        for (;;) {
            if (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1u;
                cand = jb + (uint32_t)b;
                return true;
            }
            if (j < je) { cand = j++; return true; }
            if (!live) return false;
            const int e = __ffs(live) - 1;
            live &= live - 1u;
            jb = tab[(e >> 1) * ts] + ((uint32_t)(e & 1) << 5);
            const uint32_t w = tab[(9 + e) * ts];
            if ((full >> e) & 1u) { j = jb; je = jb + w; }
            else bits = w;
        }
    }
};

// Walk of every candidate of the 27 cells, flattened across the 9 rows.
struct RangeWalk {
    const DevParams& P;
    const uint32_t* __restrict__ start;
    uint32_t cell_base, delta;
    int3 g;
    int r;
    uint32_t j, je;
    __device__ __forceinline__ RangeWalk(const DevParams& P_, const uint32_t* __restrict__ start_, uint32_t cb,
                                         uint32_t delta_, int3 g_)
        : P(P_), start(start_), cell_base(cb), delta(delta_), g(g_), r(-1), j(0), je(0) {}
    __device__ __forceinline__ bool next(uint32_t& cand) {
        for (;;) {
            if (j < je) { cand = j++; return true; }
            if (++r >= 9) return false;
            uint32_t jb;
            if (!row_range(P, start, cell_base, delta, g, r, jb, je)) { j = je = 0; continue; }
            j = jb;
        }
    }
};

// Tile scheduling of the scene-aware kernels.  With tile_ctr == nullptr each
// block runs tile blockIdx.x; otherwise the launch is persistent (a few
// blocks per SM) and blocks take tiles in turn from an atomic counter, which
// balances scenes of uneven size.  body(tile) is called by every thread of
// the block; a thread leaves a tile by returning from body.
template <class Body>
__device__ __forceinline__ void for_each_tile(const uint4* __restrict__ tiles, uint32_t ntiles,
                                              uint32_t* __restrict__ tile_ctr, Body&& body) {
    if (tile_ctr == nullptr) {
        if (blockIdx.x < ntiles) body(tiles[blockIdx.x]);
        return;
    }
    __shared__ uint32_t s_tile;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1u);
        __syncthreads();
        const uint32_t ti = s_tile;
        __syncthreads();
        if (ti >= ntiles) break;
        body(tiles[ti]);
    }
}

// Counter-based generator for lattice jitter: splitmix64 (Steele, Lea and
// Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014).
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// Uniform float in [0,1) from the top 24 bits of draw `ctr` of stream `seed`.
__host__ __device__ __forceinline__ float uniform01(uint64_t seed, uint64_t ctr) {
    const uint64_t z = splitmix64(seed ^ (ctr * 0xD1B54A32D192ED03ull));
    return (float)(uint32_t)(z >> 40) * (1.0f / 16777216.0f);
}

}  // namespace sph
