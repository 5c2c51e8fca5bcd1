// sm_103a kernels of the WCSPH substep.
//
// One substep (the body of FluidSystem::advance, fluidsystem.cu:301-398) is:
//   [k_hash: only when no force pass hashed the state] -> scan (one pass)
//   -> k_scatter -> k_rank_gather
//   -> k_density (+ the previous substep's XSPH update) -> [k_normals]
//   -> k_force_integrate [-> k_xsph, for scenes that do not defer XSPH]
// Every kernel is scene-aware: a launch covers the tiles of all live scenes,
// so the plain step is the batched step with one scene.
//
// State buffers (float4 per particle, slots indexed by the arena):
//   P0,V0,A0  state between substeps (P0.w = density of the last substep)
//   V2, okey  post-integration velocity and cell of the last substep, for a
//             scene whose XSPH update is pending (pend[scene] != 0)
//   P1,V1,A1  state gathered into cell order (with a pending update, V1.w
//             holds the gathered okey bits)
//   S         (rho, p, c^2, 1/rho^2) per sorted slot
//   Vc        cell-ordered velocities with the pending XSPH update applied
//   N         surface normals (only when a scene has surface tension)
#include <cuda_runtime.h>
#include <stdint.h>
#include "sph_types.h"
#include "sph_device.cuh"
#include "sph_kernels.h"

namespace sph {

// ---------------------------------------------------------------------------
// Spatial hash + cell counts (hash.cu:10-27 and the fill at
// fluidsystem.cu:304-306).  Equal keys inside a warp are combined with
// __match_any_sync so one atomic serves each group; the slot a particle gets
// inside its cell is provisional (atomic order) and is made stable by
// k_rank_gather.  For a scene with a pending XSPH update, a particle whose
// cell differs from the one recorded by the last force pass gets the
// SPH_OKEY_MOVED flag there (the density pass's fast adjacency test).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(SPH_TILE) k_hash(const DevParams* __restrict__ params,
                                                   const DevScene* __restrict__ scenes,
                                                   const uint4* __restrict__ tiles,
                                                   const float4* __restrict__ P, uint32_t* __restrict__ count,
                                                   uint32_t* __restrict__ key, uint32_t* __restrict__ slot,
                                                   const uint32_t* __restrict__ pend, uint32_t* __restrict__ okey,
                                                   uint32_t* __restrict__ status) {
    const uint4 t = tiles[blockIdx.x];
    if (threadIdx.x >= t.z) return;
    const uint32_t i = t.y + threadIdx.x;
    const DevScene sc = scenes[t.x];
    const DevParams& pp = params[t.x];
    const float4 p = P[i];
    const int3 gc = grid_of(pp, p.x, p.y, p.z);
    const bool inside = grid_inside(pp, gc);
    const uint32_t local = inside ? (uint32_t)gc.x + (uint32_t)gc.y * pp.gx + (uint32_t)gc.z * pp.gxy : pp.ncells;
    if (__ldg(pend + t.x) != 0u) {
        const uint32_t o = okey[i];
        if (o != SPH_OKEY_NULL && (!inside || (o & ~SPH_OKEY_MOVED) != pack_cell(gc))) okey[i] = o | SPH_OKEY_MOVED;
    }
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) atomicOr(status, SPH_STATUS_NONFINITE);
    const uint32_t gkey = sc.cell_base + local;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned active = __activemask();
    const unsigned peers = __match_any_sync(active, gkey);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(&count[gkey], (uint32_t)__popc(peers));
    base = __shfl_sync(active, base, leader);
    key[i] = local;
    slot[i] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// ---------------------------------------------------------------------------
// Exclusive scan of cell counts -> cell starts (fluidsystem.cu:316).
// Reduce-then-scan: 4096 counts per tile.
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
static_assert(SCAN_TILE == (int)kScanTileCells, "scan tile size");

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += u;
    }
    return v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t* __restrict__ in, uint32_t n,
                                                              uint32_t* __restrict__ sums) {
    const uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const uint32_t idx = base + k;
        if (idx < n) s += in[idx];
    }
    __shared__ uint32_t red[SCAN_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31u) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t w = (threadIdx.x < SCAN_THREADS / 32) ? red[threadIdx.x] : 0u;
        for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
        if (threadIdx.x == 0) sums[blockIdx.x] = w;
    }
}

// Single block: exclusive scan of up to kScanRawMaxTiles tile sums, in place.
__global__ void __launch_bounds__(1024) k_scan_top(uint32_t* __restrict__ sums, uint32_t nt) {
    constexpr int ITEMS = 32;
    static_assert(ITEMS * 1024 == (int)kScanRawMaxTiles, "k_scan_top capacity");
    uint32_t v[ITEMS];
    const uint32_t base = threadIdx.x * ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        v[k] = (base + k < nt) ? sums[base + k] : 0u;
        s += v[k];
    }
    __shared__ uint32_t warp_tot[32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_incl_scan(s);
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = warp_tot[lane];
        const uint32_t wi = warp_incl_scan(w);
        warp_tot[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = warp_tot[warp] + inc - s;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        if (base + k < nt) sums[base + k] = run;
        run += v[k];
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(const uint32_t* __restrict__ in, uint32_t n,
                                                            const uint32_t* __restrict__ sums,
                                                            uint32_t* __restrict__ out) {
    const uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const uint32_t idx = base + k;
        v[k] = (idx < n) ? in[idx] : 0u;
        s += v[k];
    }
    __shared__ uint32_t warp_tot[SCAN_THREADS / 32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_incl_scan(s);
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = (lane < SCAN_THREADS / 32) ? warp_tot[lane] : 0u;
        const uint32_t wi = warp_incl_scan(w);
        if (lane < SCAN_THREADS / 32) warp_tot[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = sums[blockIdx.x] + warp_tot[warp] + inc - s;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const uint32_t idx = base + k;
        if (idx < n) out[idx] = run;
        run += v[k];
        if (idx + 1 == n) out[n] = run;   // total after the last cell
    }
}

// Single-pass form of the same scan, used by the substep: decoupled
// look-back (Merrill and Garland, "Single-pass Parallel Prefix Scan with
// Decoupled Look-back", NVIDIA technical report NVR-2016-002).  Each tile
// publishes its aggregate, then adds the aggregates of the tiles before it
// until it meets one that has published its inclusive prefix, and publishes
// its own.  A descriptor is one 64-bit word (flag << 32 | value), so flag and
// value are read together.  desc[0] hands out tile numbers in the order the
// blocks start, so every tile waited on belongs to a block that is already
// running and waits only on tiles before it; the waits are bounded all the
// same (SPH_STATUS_SCAN_TIMEOUT, the outputs are then invalid).
//
// With `zero` set the kernel also leaves every count it read at zero: the
// next substep's hash (fused into the force pass) adds into them, which
// otherwise needs a memset of the whole count array.
constexpr unsigned long long SCAN_AGG = 1ull << 32;
constexpr unsigned long long SCAN_PRE = 2ull << 32;
constexpr uint32_t SCAN_SPIN_LIMIT = 1u << 22;   // the default limit (StepArgs.scan_spin_limit = 0)

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_single(uint32_t* __restrict__ in, uint32_t n,
                                                              unsigned long long* __restrict__ desc,
                                                              uint32_t* __restrict__ out,
                                                              uint32_t* __restrict__ status, uint32_t zero,
                                                              uint32_t spin_limit, uint32_t vec_ok) {
    __shared__ uint32_t s_tile, s_prefix, s_total;
    __shared__ uint32_t warp_tot[SCAN_THREADS / 32];
    if (threadIdx.x == 0) s_tile = atomicAdd(reinterpret_cast<unsigned int*>(desc), 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    // 16 counts in four 128-bit accesses, when `in` and `out` are 16-byte
    // aligned (a scene's own range may start anywhere)
    const bool whole = vec_ok && base + SCAN_ITEMS <= n;
    uint32_t v[SCAN_ITEMS];
    // each count is read (and, with `zero`, cleared at the end) by this thread alone
    if (whole) {
        const uint4* p4 = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
        for (int q = 0; q < SCAN_ITEMS / 4; ++q) {
            const uint4 w = p4[q];
            v[4 * q] = w.x; v[4 * q + 1] = w.y; v[4 * q + 2] = w.z; v[4 * q + 3] = w.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) v[k] = (base + k < n) ? in[base + k] : 0u;
    }
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) s += v[k];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_incl_scan(s);
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = (lane < SCAN_THREADS / 32) ? warp_tot[lane] : 0u;
        const uint32_t wi = warp_incl_scan(w);
        if (lane < SCAN_THREADS / 32) warp_tot[lane] = wi - w;
        if (lane == 31) s_total = wi;
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t agg = s_total;
        uint32_t excl = 0;
        if (tile == 0) {
            if (lane == 0) st_relaxed_u64(desc + 1, SCAN_PRE | agg);
        } else {
            if (lane == 0) st_relaxed_u64(desc + 1 + tile, SCAN_AGG | agg);
            int j = (int)tile - 1;   // lane l reads tile j - l
            for (;;) {
                const int idx = j - (int)lane;
                unsigned long long d = SCAN_PRE;   // before tile 0: an empty prefix
                if (idx >= 0) {
                    uint32_t spins = 0;
                    d = ld_relaxed_u64(desc + 1 + idx);
                    while ((d >> 32) == 0ull) {
                        if (++spins > spin_limit) {
                            atomicOr(status, SPH_STATUS_SCAN_TIMEOUT);
                            d = SCAN_PRE;
                            break;
                        }
                        __nanosleep(32);
                        d = ld_relaxed_u64(desc + 1 + idx);
                    }
                }
                const unsigned pre = __ballot_sync(0xffffffffu, (d >> 32) == 2ull);
                const int stop = pre ? __ffs(pre) - 1 : 31;   // lanes 0..stop contribute
                uint32_t val = ((int)lane <= stop) ? (uint32_t)d : 0u;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
                excl += val;
                if (pre) break;
                j -= 32;
            }
            if (lane == 0) st_relaxed_u64(desc + 1 + tile, SCAN_PRE | (excl + agg));
        }
        if (lane == 0) s_prefix = excl;
    }
    __syncthreads();
    uint32_t run = s_prefix + warp_tot[warp] + inc - s;
    if (whole) {
        uint4* o4 = reinterpret_cast<uint4*>(out + base);
#pragma unroll
        for (int q = 0; q < SCAN_ITEMS / 4; ++q) {
            uint4 w;
            w.x = run; run += v[4 * q];
            w.y = run; run += v[4 * q + 1];
            w.z = run; run += v[4 * q + 2];
            w.w = run; run += v[4 * q + 3];
            o4[q] = w;
        }
        if (base + SCAN_ITEMS == n) out[n] = run;   // total after the last cell
        if (zero) {
            uint4* z4 = reinterpret_cast<uint4*>(in + base);
#pragma unroll
            for (int q = 0; q < SCAN_ITEMS / 4; ++q) z4[q] = make_uint4(0u, 0u, 0u, 0u);
        }
    } else {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            const uint32_t idx = base + k;
            if (idx < n) out[idx] = run;
            run += v[k];
            if (idx + 1 == n) out[n] = run;
            if (zero && idx < n) in[idx] = 0u;
        }
    }
}

// The cell starts are invalid once a wait of the scan ran out, and the cell
// order is incomplete once the rank pass met a cell of more than
// SPH_MAX_CELL_OCC particles (it writes no slot of that cell): every pass
// that indexes with them returns at once, and the step reports SPH_ETIMEOUT
// or SPH_ECELL with the particles as they were before the failed substep.
// Each block tests once, at its start; only the rank pass raises a bit this
// tests while later passes could see it, and its output is dropped anyway.
__device__ __forceinline__ bool step_failed(const uint32_t* status) {
    return (__ldcg(status) & (SPH_STATUS_SCAN_TIMEOUT | SPH_STATUS_CELL_OVERFLOW)) != 0u;
}

// ---------------------------------------------------------------------------
// Scatter: provisional slot of each particle in cell order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(SPH_TILE) k_scatter(const DevScene* __restrict__ scenes,
                                                      const uint4* __restrict__ tiles,
                                                      const uint32_t* __restrict__ start,
                                                      const uint32_t* __restrict__ key,
                                                      const uint32_t* __restrict__ slot,
                                                      uint32_t* __restrict__ tmp,
                                                      const uint32_t* __restrict__ status) {
    if (step_failed(status)) return;
    const uint4 t = tiles[blockIdx.x];
    if (threadIdx.x >= t.z) return;
    const uint32_t i = t.y + threadIdx.x;
    const DevScene sc = scenes[t.x];
    const uint32_t s0 = __ldg(start + sc.cell_base);
    const uint32_t c = sc.cell_base + key[i];
    tmp[sc.part_base + (__ldg(start + c) - s0) + slot[i]] = i;
}

// ---------------------------------------------------------------------------
// Stable rank inside the cell + gather into cell order.  thrust::sort_by_key
// over u32 keys (fluidsystem.cu:309-313) is a stable radix sort: within a cell
// particles keep their current order.  Each sorted slot's final position is
// the cell start plus the number of cell members with a smaller current
// index, which reproduces that permutation exactly.
// A scene whose last XSPH update is still pending (pend[scene] != 0) has its
// post-integration velocities in V2 and its previous cells in okey: those
// are gathered (the density pass applies the XSPH update); otherwise V0.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(SPH_TILE) k_rank_gather(const DevScene* __restrict__ scenes,
                                                          const uint4* __restrict__ tiles,
                                                          const uint32_t* __restrict__ start,
                                                          const uint32_t* __restrict__ key,
                                                          const uint32_t* __restrict__ tmp,
                                                          const float4* __restrict__ P0,
                                                          const float4* __restrict__ V0,
                                                          const float4* __restrict__ A0,
                                                          const float4* __restrict__ V2,
                                                          const uint32_t* __restrict__ okey,
                                                          const uint32_t* __restrict__ pend,
                                                          float4* __restrict__ P1, float4* __restrict__ V1,
                                                          float4* __restrict__ A1,
                                                          uint32_t* __restrict__ perm,
                                                          uint32_t* __restrict__ status) {
    if (step_failed(status)) return;
    const uint4 t = tiles[blockIdx.x];
    if (threadIdx.x >= t.z) return;
    const uint32_t g = t.y + threadIdx.x;
    const DevScene sc = scenes[t.x];
    const bool pending = __ldg(pend + t.x) != 0u;
    const uint32_t i = tmp[g];
    const uint32_t s0 = __ldg(start + sc.cell_base);
    const uint32_t c = sc.cell_base + __ldg(key + i);
    const uint32_t b = sc.part_base + (__ldg(start + c) - s0);
    const uint32_t e = sc.part_base + (__ldg(start + c + 1) - s0);
    if (e - b > SPH_MAX_CELL_OCC) {
        atomicOr(status, SPH_STATUS_CELL_OVERFLOW);
        return;
    }
    uint32_t rank = 0;
    for (uint32_t m = b; m < e; ++m) rank += (__ldg(tmp + m) < i) ? 1u : 0u;
    const uint32_t f = b + rank;
    perm[f] = i;
    P1[f] = P0[i];
    float4 v = pending ? V2[i] : V0[i];
    // the cell of the last substep travels with the velocity (w lane) to the
    // density pass's XSPH update, which loads both together
    if (pending) v.w = __uint_as_float(__ldg(okey + i));
    V1[f] = v;
    A1[f] = A0[i];
}

// ---------------------------------------------------------------------------
// Density + Tait EOS (computeDensity, fluidphysics.cu:8-84), in two phases.
//
// Phase 1 scans the candidates of the 27 cells, 32 at a time, with the
// distance test alone and records a bit per candidate within h (density
// pairs, j != i) and, with SKIN, within the skin radius.  The words go to the
// neighbour masks of the later passes (SPH_MASK_SKIN rows for rows of up to
// 32 candidates; SPH_MASK_EXACT rows, two words per row of up to 64) and to a
// row table in shared memory (build_row_table's layout).  Coincident pairs
// (r^2 <= eps) stay in the words: the density sum and XSPH take them, and the
// normal and force passes drop them with their own r^2 > eps test.  Phase 2
// walks that table and does the kernel arithmetic for the density pairs only
// (about one candidate in six), so a warp no longer runs the neighbour path
// on every candidate that any of its lanes accepts.  Rows longer than 64
// candidates are not scanned in phase 1; phase 2 walks them in full with the
// test.  Both phases visit candidates in the same order (rows z outer, then
// y, then slots, the row's cells x ascending), so the sum follows phase 1's
// candidate order; the reference's loop runs the cells x outer and z inner
// (fluidphysics.cu:29-33), the same terms in another order.  WALK selects
// phase 1's loop: flattened across the
// rows (0) or one loop per row with four candidates in flight, two per
// 256-bit load (1); the words are
// the same.
//
// Deferred XSPH.  For a scene whose previous substep ended without its XSPH
// update (pend[scene] != 0), P1 holds that substep's post-integration
// positions (w = its densities), V1 its post-integration velocities with, in
// the w lane, the cells the particles were sorted into then (okey bits).  The reference's update
// (correctVelocityXSPH, fluidphysics.cu:355-409) sums over pairs with
// r^2 <= h^2 at these positions whose previous cells are adjacent (its cell
// lists were those of the previous sort); every such pair is within h now, so
// phase 2 meets all of them, and the previous-cell test keeps exactly the
// reference's pairs.  The poly6 weight is the one the density sum uses.  The
// corrected velocity goes to Vc, which the force pass reads; without a
// pending update Vc = V1.
// ---------------------------------------------------------------------------
// Two consecutive cell-ordered positions in one 256-bit load: the slot must
// be even (32-byte aligned from the 256-byte aligned arena).  The positions
// are not written during the pass that reads them.
__device__ __forceinline__ void ld_pos_pair(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

#ifndef DENSITY_MINB
#define DENSITY_MINB 4
#endif
// SPLIT (with WALK == 1, no SKIN, one block per tile): three threads per
// particle share phase 1, thread q of the particle taking rows 3q..3q+2; its
// words and row-table entries are per row, so phase 1 writes exactly what
// one thread would.  After a barrier the first thread runs phase 2 over the
// whole table.  A small scene's pass lasts as long as one thread's walk, and
// the split shortens the candidate scan's share of it threefold.
template <int WALK, bool SKIN, bool SPLIT = false>
__global__ void __launch_bounds__(SPLIT ? 3 * SPH_TILE : SPH_TILE, SPLIT ? 1 : DENSITY_MINB)
k_density(const DevParams* __restrict__ params,
                                                      const DevScene* __restrict__ scenes,
                                                      const uint4* __restrict__ tiles,
                                                      const uint32_t* __restrict__ start,
                                                      const float4* __restrict__ P1, float4* __restrict__ S,
                                                      uint32_t* __restrict__ mask, size_t mask_stride,
                                                      const float4* __restrict__ V1,
                                                      const uint32_t* __restrict__ pend, float4* __restrict__ Vc,
                                                      uint32_t* __restrict__ nbr_out, uint32_t ntiles,
                                                      uint32_t* __restrict__ tile_ctr,
                                                      const uint32_t* __restrict__ status) {
  static_assert(!SPLIT || (WALK == 1 && !SKIN), "the split scan is the per-row scan without skin words");
  extern __shared__ uint32_t s_rows[];
  if (step_failed(status)) return;
  for_each_tile(tiles, ntiles, tile_ctr, [&](const uint4 t) {
    // particle li of the tile; with SPLIT, part q of its phase 1.  Every
    // thread of a split block reaches the barrier after phase 1.
    const uint32_t ts = SPLIT ? blockDim.x / 3u : blockDim.x;
    const uint32_t part = SPLIT ? threadIdx.x / ts : 0u;
    const uint32_t li = SPLIT ? threadIdx.x - part * ts : threadIdx.x;
    if (!SPLIT && li >= t.z) return;
    const bool act = !SPLIT || li < t.z;
    const uint32_t k = t.y + li;
    const DevScene sc = scenes[t.x];
    const DevParams& pp = params[t.x];
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f), vi = p;
    if (act) {
        p = P1[k];
        vi = V1[k];
    }
    const int3 g = grid_of(pp, p.x, p.y, p.z);
    const bool work = act && grid_inside(pp, g);
    if (act && !work) {
        if (part == 0u) {
            S[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            Vc[k] = make_float4(vi.x, vi.y, vi.z, 0.f);
            if (nbr_out) nbr_out[k] = 0;
        }
        if (!SPLIT) return;
    }
    const uint32_t delta = sc.part_base - __ldg(start + sc.cell_base);
    // the skin-radius words serve only the per-substep XSPH pass
    const float h2 = pp.h2, skin2 = SKIN ? pp.skin2 : pp.h2, eps = pp.eps;
    uint32_t* tab = s_rows + li;
    uint32_t live = 0u, full = 0u;
    // rows of this thread's phase 1
    constexpr int kRows = SPLIT ? 3 : 9;
    const int r0 = SPLIT ? 3 * (int)part : 0;

    // ---- phase 1: distance test of every candidate ----
    auto visit = [&](const float4& q, uint32_t bit, uint32_t& dm, uint32_t& sm) {
        const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        const float rr = dot3(dx, dy, dz, dx, dy, dz);
        if (rr <= h2) dm |= bit;
        if (SKIN && rr <= skin2) sm |= bit;
    };
    // Two candidates at once with the packed FP32 instructions of sm_100-class
    // GPUs (add/mul/fma.rn.f32x2): each component is rounded exactly as the
    // scalar operation, so r^2 (dot3's fusion order) is the same to the bit.
    const float2 px2 = make_float2(p.x, p.x), py2 = make_float2(p.y, p.y), pz2 = make_float2(p.z, p.z);
    auto visit2 = [&](const float4& q0, const float4& q1, uint32_t bit, uint32_t& dm, uint32_t& sm) {
        const float2 dx = __fadd2_rn(px2, make_float2(-q0.x, -q1.x));
        const float2 dy = __fadd2_rn(py2, make_float2(-q0.y, -q1.y));
        const float2 dz = __fadd2_rn(pz2, make_float2(-q0.z, -q1.z));
        const float2 rr = __ffma2_rn(dz, dz, __ffma2_rn(dx, dx, __fmul2_rn(dy, dy)));
        if (rr.x <= h2) dm |= bit;
        if (rr.y <= h2) dm |= bit << 1;
        if (SKIN && rr.x <= skin2) sm |= bit;
        if (SKIN && rr.y <= skin2) sm |= bit << 1;
    };
    // The words of chunk c of row r (bit b = candidate jb0 + 32c + b) minus
    // the particle itself, stored to the masks and the row table.
    auto close_chunk = [&](int r, uint32_t c, uint32_t jb0, uint32_t len, uint32_t dm, uint32_t sm) {
        const uint32_t so = k - (jb0 + 32u * c);
        const uint32_t notself = (so < 32u) ? ~(1u << so) : ~0u;
        dm &= notself;
        if (SKIN && len <= 32u) mask[(size_t)(SPH_MASK_SKIN + r) * mask_stride + k] = sm & notself;
        mask[(size_t)(SPH_MASK_EXACT + 2 * r + c) * mask_stride + k] = dm;
        if (c == 0u) tab[r * ts] = jb0;
        tab[(9 + 2 * r + c) * ts] = dm;
        if (dm) live |= 1u << (2 * r + c);
    };
    // A row longer than 64 candidates: no words, phase 2 tests every candidate.
    auto long_row = [&](int r, uint32_t jb0, uint32_t len) {
        tab[r * ts] = jb0;
        tab[(9 + 2 * r) * ts] = len;
        full |= 1u << (2 * r);
        live |= 1u << (2 * r);
    };
    // The 9 row ranges, loaded together (18 independent loads) into the row
    // table; a row's end sits in its first word's entry until the scan of
    // the row replaces it.
    uint32_t rows = 0u;
#pragma unroll
    for (int rr = 0; rr < kRows; ++rr) {
        const int r = r0 + rr;
        uint32_t jb0, je0;
        if ((!SPLIT || work) && row_range(pp, start, sc.cell_base, delta, g, r, jb0, je0)) {
            rows |= 1u << r;
            tab[r * ts] = jb0;
            tab[(9 + 2 * r) * ts] = je0;
        }
    }
    if (WALK == 1) {
#pragma unroll 1
        for (int rr = 0; rr < kRows; ++rr) {
            const int r = r0 + rr;
            if (!((rows >> r) & 1u)) continue;
            const uint32_t jb0 = tab[r * ts], je0 = tab[(9 + 2 * r) * ts];
            const uint32_t len = je0 - jb0;
            if (len > SPH_WIDE_ROW) { long_row(r, jb0, len); continue; }
            uint32_t cb = jb0, c = 0u;
            do {
                const uint32_t ce = min(cb + 32u, je0);
                uint32_t dm = 0u, sm = 0u, bit = 1u;
                uint32_t jj = cb;
                // from an even slot on, two candidates per 256-bit load (an
                // empty row runs this body once, with cb == ce: no candidate)
                if (jj < ce && (jj & 1u) != 0u) {
                    visit(__ldg(P1 + jj), bit, dm, sm);
                    bit <<= 1;
                    ++jj;
                }
                for (; jj + 4u <= ce; jj += 4u) {
                    float4 q0, q1, q2, q3;
                    ld_pos_pair(P1 + jj, q0, q1);
                    ld_pos_pair(P1 + jj + 2u, q2, q3);
                    visit2(q0, q1, bit, dm, sm);
                    visit2(q2, q3, bit << 2, dm, sm);
                    bit <<= 4;
                }
                if (jj + 2u <= ce) {
                    float4 q0, q1;
                    ld_pos_pair(P1 + jj, q0, q1);
                    visit2(q0, q1, bit, dm, sm);
                    bit <<= 2;
                    jj += 2u;
                }
                if (jj < ce) visit(__ldg(P1 + jj), bit, dm, sm);
                close_chunk(r, c, jb0, len, dm, sm);
                cb += 32u;
                ++c;
            } while (cb < je0);
        }
    } else {
        // one loop across all 9 rows and their chunks, so lanes do not wait at
        // row ends
        int r = -1;
        uint32_t jb = 0, je = 0, j = 0, cend = 0, c = 0, len = 0, dm = 0u, sm = 0u, bit = 0u;
        bool valid = false;
        for (;;) {
            if (j >= cend) {
                if (valid) {
                    close_chunk(r, c, jb, len, dm, sm);
                    if (j < je) {   // the row's second chunk
                        ++c;
                        cend = min(j + 32u, je);
                        dm = sm = 0u;
                        bit = 1u;
                        continue;
                    }
                }
                if (++r >= 9) break;
                valid = ((rows >> r) & 1u) != 0u;
                jb = valid ? tab[r * ts] : 0u;
                je = valid ? tab[(9 + 2 * r) * ts] : 0u;
                len = je - jb;
                if (valid && len > SPH_WIDE_ROW) {
                    long_row(r, jb, len);
                    valid = false;
                    j = cend = 0;
                    continue;
                }
                c = 0u;
                j = jb;
                cend = min(jb + 32u, je);
                dm = sm = 0u;
                bit = 1u;
                continue;
            }
            visit(__ldg(P1 + j), bit, dm, sm);
            bit <<= 1;
            ++j;
        }
    }

    if constexpr (SPLIT) {
        // the parts' row bits are disjoint: the first thread takes their union
        __shared__ uint32_t s_bits[2 * 3 * SPH_TILE];
        s_bits[2 * threadIdx.x] = live;
        s_bits[2 * threadIdx.x + 1] = full;
        __syncthreads();
        if (part != 0u || !work) return;
        live = s_bits[2 * li] | s_bits[2 * (ts + li)] | s_bits[2 * (2 * ts + li)];
        full = s_bits[2 * li + 1] | s_bits[2 * (ts + li) + 1] | s_bits[2 * (2 * ts + li) + 1];
    }

    // ---- phase 2: the density pairs, in candidate order ----
    const float h = pp.h, mass = pp.mass, c6 = pp.poly6, two_m = pp.two_mass;
    float sum = 0.0f;
    uint32_t cnt = 0;
    // deferred XSPH of the previous substep (only for particles that had a cell then)
    const uint32_t oi = (__ldg(pend + t.x) != 0u) ? __float_as_uint(vi.w) : SPH_OKEY_NULL;
    const bool xs = oi != SPH_OKEY_NULL;
    // XSPH sums: x and y packed (f32x2), z alone
    float2 axy = make_float2(0.f, 0.f);
    float az = 0.f;
    const float2 mvixy = make_float2(-vi.x, -vi.y);
    TableWalk walk(tab, ts, live, full);
    uint32_t j;
    while (walk.next(j)) {
        // the pair's XSPH operands (velocity, and its last cell in the w
        // lane) are loaded with its position, before any test, so that the
        // two latencies overlap
        const float4 q = __ldg(P1 + j);
        float4 vj = make_float4(0.f, 0.f, 0.f, 0.f);
        if (xs) vj = __ldg(V1 + j);
        const uint32_t oj = __float_as_uint(vj.w);
        const float2 dxy = __fadd2_rn(make_float2(p.x, p.y), make_float2(-q.x, -q.y));
        const float dx = dxy.x, dy = dxy.y, dz = p.z - q.z;
        const float rr = dot3(dx, dy, dz, dx, dy, dz);
        // true for every recorded bit; the test matters in rows walked in full
        if (rr <= h2 && j != k) {
            const float rd = sqrtf(rr);
            const float x = fmaf(-rd, rd, h2);
            const float w = (rd >= h) ? 0.0f : c6 * (x * x * x);
            sum = fmaf(mass, w, sum);
            cnt++;
            if (xs) {
                const float rs = p.w + q.w;   // the previous substep's densities
                if (rs > eps && cells_adjacent_fast(oi, oj)) {
                    const float coeff = w * __fdividef(two_m, rs);
                    axy = __ffma2_rn(make_float2(coeff, coeff), __fadd2_rn(make_float2(vj.x, vj.y), mvixy), axy);
                    az = fmaf(coeff, vj.z - vi.z, az);
                }
            }
        }
    }
    const float d = fabsf(sdf(pp, p.x, p.y, p.z));
    float corr = sum;
    if (d < pp.h) corr = fmaf(pp.rest_density, 1.0f - boundary_density(pp, d), corr);
    const float rho = (sum == 0.0f) ? pp.rest_density : corr;
    const float ratio = corr * pp.inv_rest_density;
    const float prs = (corr == 0.0f) ? 0.0f : pp.eos_k * (powf(ratio, pp.gamma) - 1.0f);
    const float cs = pp.gas_constant * powf(ratio, pp.gamma - 1.0f);
    // w = 1/rho^2, used by the force pass for p_j/rho_i^2 + p_i/rho_j^2
    S[k] = make_float4(rho, prs, cs, 1.0f / (rho * rho));
    Vc[k] = xs ? make_float4(fmaf(pp.xsph, axy.x, vi.x), fmaf(pp.xsph, axy.y, vi.y), fmaf(pp.xsph, az, vi.z), 0.f)
               : make_float4(vi.x, vi.y, vi.z, 0.f);
    if (nbr_out) nbr_out[k] = cnt;
  });
}

// ---------------------------------------------------------------------------
// Surface normals (computeNormals, fluidphysics.cu:154-210).  Only launched
// for scenes with surface tension: with sigma == 0 the normals enter the
// force only through sigma * (...), which is exactly zero.  TABLE walks a row
// table in shared memory as the force pass does; same neighbours, same order.
// ---------------------------------------------------------------------------
template <bool TABLE>
__global__ void __launch_bounds__(SPH_TILE) k_normals(const DevParams* __restrict__ params,
                                                      const DevScene* __restrict__ scenes,
                                                      const uint4* __restrict__ tiles,
                                                      const uint32_t* __restrict__ start,
                                                      const float4* __restrict__ P1,
                                                      const float4* __restrict__ S,
                                                      const uint32_t* __restrict__ mask, size_t mask_stride,
                                                      float4* __restrict__ N, uint32_t ntiles,
                                                      uint32_t* __restrict__ tile_ctr,
                                                      const uint32_t* __restrict__ status) {
  if (step_failed(status)) return;
  for_each_tile(tiles, ntiles, tile_ctr, [&](const uint4 t) {
    const DevParams& pp = params[t.x];
    if (!(pp.flags & 1u)) return;
    if (threadIdx.x >= t.z) return;
    const uint32_t k = t.y + threadIdx.x;
    const DevScene sc = scenes[t.x];
    const float4 p = P1[k];
    const int3 g = grid_of(pp, p.x, p.y, p.z);
    if (!grid_inside(pp, g)) {
        N[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const uint32_t delta = sc.part_base - __ldg(start + sc.cell_base);
    // x and y packed (f32x2, rounded per component as the scalar operations), z alone
    float2 sxy = make_float2(0.f, 0.f);
    float sz = 0.f;
    const float2 pxy = make_float2(p.x, p.y);
    // m gradPoly6(r) rvec / (rho_j r) = m c (h^2 - r^2)^2 rvec / rho_j: the
    // factor r of gradPoly6 cancels the 1/r; h^2 - r^2 is formed from the
    // rounded root r as gradPoly6 forms it (it cancels near r = h)
    const float mc = pp.mass * pp.grad_poly6;
    const float h2 = pp.h2, eps = pp.eps, h = pp.h;
    auto run = [&](auto& walk) {
        uint32_t j;
        while (walk.next(j)) {
            const float4 q = __ldg(P1 + j);
            const float rhoj = __ldg(&S[j].x);
            const float2 rxy = __fadd2_rn(pxy, make_float2(-q.x, -q.y));
            const float rx = rxy.x, ry = rxy.y, rz = p.z - q.z;
            const float r2 = dot3(rx, ry, rz, rx, ry, rz);
            if (r2 <= h2 && r2 > eps && j != k && rhoj > eps) {
                const float r = sqrtf(r2);
                const float x = fmaf(-r, r, h2);
                const float s = (r >= h) ? 0.0f : __fdividef(mc * (x * x), rhoj);
                sxy = __ffma2_rn(make_float2(s, s), rxy, sxy);
                sz = fmaf(s, rz, sz);
            }
        }
    };
    // exact neighbours recorded by the density pass (SPH_MASK_EXACT words)
    if constexpr (TABLE) {
        extern __shared__ uint32_t s_rows[];
        uint32_t live, full;
        build_row_table(pp, start, sc.cell_base, delta, g, mask + SPH_MASK_EXACT * mask_stride, mask_stride, k,
                        s_rows + threadIdx.x, blockDim.x, live, full);
        TableWalk walk(s_rows + threadIdx.x, blockDim.x, live, full);
        run(walk);
    } else {
        WideMaskWalk walk(pp, start, sc.cell_base, delta, g, mask + SPH_MASK_EXACT * mask_stride, mask_stride, k);
        run(walk);
    }
    N[k] = make_float4(pp.h * sxy.x, pp.h * sxy.y, pp.h * sz, 0.f);
  });
}

// ---------------------------------------------------------------------------
// Forces (computeAllForces, fluidphysics.cu:215-352) fused with the leapfrog
// integrator and box boundary (LeapfrogIntegratorOperator,
// fluidintegrator.cu:11-70).  Reads cell-order state (P1, the velocities Vc
// of the density pass (V1 with any pending XSPH update applied) through the
// V1 argument, A1, S, N), writes the integrated state to P0 (w = density), V2,
// A0, each particle's cell to okey, and the next substep's hash of the new
// positions (key, slot, cell counts), so that substep needs no hash pass.
// The integrator sums the
// force buffers in the reference's order, which after the swapped arguments
// at fluidsystem.cu:352-364 is ((pressure + tension) + viscosity) + adhesion.
// ---------------------------------------------------------------------------
// TENSION = false is the build for launches where no scene has surface
// tension (the tension terms are then compiled out).  MINB is the register
// budget as resident blocks of 256 threads per SM: 3 (85 registers; the
// tension-free build needs 72, the tension build 80, no spills) or 4 (64
// registers, more warps per SM, a few spilled values).
template <bool TENSION, int MINB, bool TABLE>
__global__ void __launch_bounds__(SPH_TILE, MINB)
k_force_integrate(const DevParams* __restrict__ params,
                                                              const DevScene* __restrict__ scenes,
                                                              const uint4* __restrict__ tiles,
                                                              const uint32_t* __restrict__ start,
                                                              const float4* __restrict__ P1,
                                                              const float4* __restrict__ V1,
                                                              const float4* __restrict__ A1,
                                                              const float4* __restrict__ S,
                                                              const float4* __restrict__ N,
                                                              const uint32_t* __restrict__ mask, size_t mask_stride,
                                                              float4* __restrict__ P0, float4* __restrict__ V2,
                                                              float4* __restrict__ A0, uint32_t* __restrict__ maxdisp,
                                                              uint32_t* __restrict__ okey, uint32_t* __restrict__ pend,
                                                              uint32_t* __restrict__ count, uint32_t* __restrict__ key,
                                                              uint32_t* __restrict__ slot, uint32_t* __restrict__ status,
                                                              float4* __restrict__ dbg_forces, uint32_t ntiles,
                                                              uint32_t* __restrict__ tile_ctr) {
  if (step_failed(status)) return;
  for_each_tile(tiles, ntiles, tile_ctr, [&](const uint4 t) {
    // lanes holding a particle of this tile (taken before any divergence)
    const unsigned lanes = __ballot_sync(0xffffffffu, threadIdx.x < t.z);
    if (threadIdx.x >= t.z) return;
    const uint32_t k = t.y + threadIdx.x;
    const DevScene sc = scenes[t.x];
    const DevParams& pp = params[t.x];
    // the scene's XSPH update is now pending (applied by the next density
    // pass, or by k_xsph right after this pass)
    if (threadIdx.x == 0) pend[t.x] = 1u;
    const float4 pi = P1[k];
    const float4 vi = V1[k];
    const float4 si = S[k];
    const int3 g = grid_of(pp, pi.x, pi.y, pi.z);
    const bool tension = TENSION && (pp.flags & 1u) != 0u;
    const bool inside = grid_inside(pp, g);
    float fpx = 0.f, fpy = 0.f, fpz = 0.f;   // pressure
    float fvx = 0.f, fvy = 0.f, fvz = 0.f;   // "viscosity" (pressure re-added)
    float ftx = 0.f, fty = 0.f, ftz = 0.f;   // tension
    float fax = 0.f, fay = 0.f, faz = 0.f;   // adhesion
    const uint32_t delta = sc.part_base - __ldg(start + sc.cell_base);
    const float ri = si.x, pri = si.y, csi = si.z;
    float4 ni = make_float4(0.f, 0.f, 0.f, 0.f);
    if (tension && inside) ni = N[k];
    const float h2 = pp.h2, eps = pp.eps, inv_ri2 = si.w;
    // 2 rho0 / (rho_i + rho_i) of the tension sum (fluidphysics.cu:293), once per particle
    const float tden = (2.0f * pp.rest_density) / (ri + ri);
    const float sm = -pp.surface_tension * pp.mass;
    const float coh_m = -pp.mass * pp.mass;
    // per-scene constants of the pair loop, held in registers
    const float visc = pp.viscosity, hh = pp.h, visc_eps = pp.visc_eps, mass = pp.mass, gsp = pp.grad_spiky;
    // One pair: neighbour j with its position, (rho, p, c^2, 1/rho^2),
    // velocity and normal.
    auto pair = [&](uint32_t j, const float4& pj, const float4& sj, const float4& vj, const float4& nj) {
        const float rx = pj.x - pi.x, ry = pj.y - pi.y, rz = pj.z - pi.z;
        const float r2 = dot3(rx, ry, rz, rx, ry, rz);
        if (r2 <= h2 && r2 > eps && j != k && sj.x > eps) {
            // r is the correctly rounded root: h - r below cancels, and pairs at
            // r ~ h must see the reference's r; 1/r only scales (approximate)
            const float r = sqrtf(r2);
            const float inv_r = rsqrtf(r2);
            const float ux = dot3(vi.x - vj.x, vi.y - vj.y, vi.z - vj.z, -rx, -ry, -rz);
            // artificial viscosity -visc (cs_i + cs_j) mu / (rho_i + rho_j),
            // mu = h ux / (r^2 + 0.01 h^2), only for approaching pairs;
            // evaluated without a branch (finite for every pair) and selected
            const float Pv = __fdividef(-visc * (csi + sj.z) * (hh * ux), (r2 + visc_eps) * (ri + sj.x));
            const float Pi = (ux < 0.0f) ? Pv : 0.0f;
            // p_j/rho_i^2 + p_i/rho_j^2 with the reciprocals from the density pass
            const float mid = sj.y * inv_ri2 + pri * sj.w;
            const float gspk = (r >= hh) ? 0.0f : gsp * (hh - r) * (hh - r);   // grad_spiky
            const float sr = (mass * gspk) * inv_r;
            const float cx = sr * rx, cy = sr * ry, cz = sr * rz;
            fpx = fmaf(cx, mid, fpx); fpy = fmaf(cy, mid, fpy); fpz = fmaf(cz, mid, fpz);
            const float mp = mid + Pi;
            fvx = fmaf(cx, mp, fvx); fvy = fmaf(cy, mp, fvy); fvz = fmaf(cz, mp, fvz);
            if (tension) {
                // Akinci cohesion + curvature (fluidphysics.cu:291-293).  With
                // sigma == 0 the tension force is sigma * (finite sum) = 0, so
                // the term is skipped.
                const float sc2 = coh_m * cohesion_k(pp, r) * inv_r;
                const float hx = sc2 * rx, hy = sc2 * ry, hz = sc2 * rz;
                const float kx = sm * (ni.x - nj.x), ky = sm * (ni.y - nj.y), kz = sm * (ni.z - nj.z);
                ftx = fmaf(tden, hx + kx, ftx);
                fty = fmaf(tden, hy + ky, fty);
                ftz = fmaf(tden, hz + kz, ftz);
            }
        }
    };
    // The neighbour's loads are issued together, before any test, so that
    // their latencies overlap (the masks hold exact neighbours: nearly every
    // j is used).
    auto gathered = [&](uint32_t j) {
        const float4 pj = __ldg(P1 + j), sj = __ldg(S + j), vj = __ldg(V1 + j);
        float4 nj = make_float4(0.f, 0.f, 0.f, 0.f);
        if (tension) nj = __ldg(N + j);
        pair(j, pj, sj, vj, nj);
    };
    // exact neighbours recorded by the density pass (SPH_MASK_EXACT words)
    if (inside) {
        if constexpr (TABLE) {
            extern __shared__ uint32_t s_rows[];
            uint32_t live, full;
            build_row_table(pp, start, sc.cell_base, delta, g, mask + SPH_MASK_EXACT * mask_stride, mask_stride, k,
                            s_rows + threadIdx.x, blockDim.x, live, full);
            TableWalk walk(s_rows + threadIdx.x, blockDim.x, live, full);
            uint32_t j;
            while (walk.next(j)) gathered(j);
        } else {
            WideMaskWalk walk(pp, start, sc.cell_base, delta, g, mask + SPH_MASK_EXACT * mask_stride, mask_stride, k);
            uint32_t j;
            while (walk.next(j)) gathered(j);
        }
    }
    if (inside) {
        fvx = pp.viscosity * fvx; fvy = pp.viscosity * fvy; fvz = pp.viscosity * fvz;
        ftx = pp.surface_tension * ftx; fty = pp.surface_tension * fty; ftz = pp.surface_tension * ftz;
        const float z = -fminf(sdf(pp, pi.x, pi.y, pi.z), 0.0f) * 0.25f * pp.inv_particle_size;
        if (z < 1.0f) {
            const float3 nb = sdf_normal(pp, pi.x, pi.y, pi.z);
            const float denom = 1.0f / powf(1.0f - z, 3.0f);
            const float a = pp.adhesion * ri * pp.inv_rest_density * denom;
            fax = a * nb.x; fay = a * nb.y; faz = a * nb.z;
        }
    }
    if (dbg_forces) {
        dbg_forces[4 * (size_t)k + 0] = make_float4(fpx, fpy, fpz, 0.f);
        dbg_forces[4 * (size_t)k + 1] = make_float4(ftx, fty, ftz, 0.f);
        dbg_forces[4 * (size_t)k + 2] = make_float4(fax, fay, faz, 0.f);
        dbg_forces[4 * (size_t)k + 3] = make_float4(fvx, fvy, fvz, 0.f);
    }
    // ---- leapfrog integrator + boundary ----
    const float4 ai = A1[k];
    const float Fx = ((fpx + ftx) + fvx) + fax;
    const float Fy = ((fpy + fty) + fvy) + fay;
    const float Fz = ((fpz + ftz) + fvz) + faz;
    float anx = fmaf(Fx, pp.mass, pp.grav_x), any = fmaf(Fy, pp.mass, pp.grav_y), anz = fmaf(Fz, pp.mass, pp.grav_z);
    float sq = dot3(anx, any, anz, anx, any, anz);
    if (sq > pp.acc_limit2) {
        const float s = pp.acc_limit / sqrtf(sq);
        anx = anx * s; any = any * s; anz = anz * s;
    }
    float px = pi.x + fmaf(vi.x, pp.dt, (0.5f * ai.x) * pp.dtdt);
    float py = pi.y + fmaf(vi.y, pp.dt, (0.5f * ai.y) * pp.dtdt);
    float pz = pi.z + fmaf(vi.z, pp.dt, (0.5f * ai.z) * pp.dtdt);
    float vx = fmaf(0.5f * (ai.x + anx), pp.dt, vi.x);
    float vy = fmaf(0.5f * (ai.y + any), pp.dt, vi.y);
    float vz = fmaf(0.5f * (ai.z + anz), pp.dt, vi.z);
    sq = dot3(vx, vy, vz, vx, vy, vz);
    if (sq > pp.vel_limit2) {
        const float s = pp.vel_limit / sqrtf(sq);
        vx = vx * s; vy = vy * s; vz = vz * s;
    }
    const float d = sdf(pp, px, py, pz);
    if (d > -pp.particle_size) {
        const float3 nb = sdf_normal(pp, px, py, pz);
        const float s = -(d + pp.particle_size);
        px = fmaf(s, nb.x, px); py = fmaf(s, nb.y, py); pz = fmaf(s, nb.z, pz);
        const float kk = (1.0f + pp.vdamp) * dot3(nb.x, nb.y, nb.z, vx, vy, vz);
        vx = fmaf(-kk, nb.x, vx); vy = fmaf(-kk, nb.y, vy); vz = fmaf(-kk, nb.z, vz);
    }
    P0[k] = make_float4(px, py, pz, si.x);
    V2[k] = make_float4(vx, vy, vz, 0.f);
    A0[k] = make_float4(anx, any, anz, 0.f);
    // The next substep's hash (k_hash's work, on the position just written):
    // its cell key, a provisional slot from the cell count (made stable by
    // the rank pass) and the non-finite check.  The cell XSPH's cell lists
    // use is recorded with SPH_OKEY_MOVED when the particle leaves it.
    const int3 gn = grid_of(pp, px, py, pz);
    const bool inside_new = grid_inside(pp, gn);
    if (!(isfinite(px) && isfinite(py) && isfinite(pz))) atomicOr(status, SPH_STATUS_NONFINITE);
    const uint32_t local = inside_new ? (uint32_t)gn.x + (uint32_t)gn.y * pp.gx + (uint32_t)gn.z * pp.gxy : pp.ncells;
    {
        const uint32_t gkey = sc.cell_base + local;
        const unsigned lane = threadIdx.x & 31u;
        const unsigned peers = __match_any_sync(lanes, gkey);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(&count[gkey], (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        key[k] = local;
        slot[k] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
    }
    okey[k] = grid_inside(pp, g)
                  ? (pack_cell(g) | ((inside_new && pack_cell(gn) == pack_cell(g)) ? 0u : SPH_OKEY_MOVED))
                  : SPH_OKEY_NULL;
    // largest displacement of the substep in units of h (squared), for XSPH's
    // use of the neighbour masks; NaN compares above every finite value
    const float ddx = px - pi.x, ddy = py - pi.y, ddz = pz - pi.z;
    const float d2 = dot3(ddx, ddy, ddz, ddx, ddy, ddz) * pp.inv_h2;
    const uint32_t bits = (d2 != d2) ? 0x7fffffffu : __float_as_uint(d2);
    if (maxdisp) {   // only scenes with a per-substep XSPH pass use the skin masks
        const uint32_t wmax = __reduce_max_sync(lanes, bits);
        if ((threadIdx.x & 31u) == (uint32_t)(__ffs(lanes) - 1)) atomicMax(maxdisp, wmax);
    }
  });
}

// One XSPH pair term (fluidphysics.cu:392-401).
__device__ __forceinline__ void xsph_pair(const float4* __restrict__ P0, const float4* __restrict__ V2, uint32_t j,
                                          uint32_t k, const float4& pi, const float4& vi, float h2, float h, float c6,
                                          float two_m, float eps, float& sx, float& sy, float& sz) {
    const float4 q = __ldg(P0 + j);
    const float4 vj = __ldg(V2 + j);   // issued with the position: most candidates are neighbours
    const float dx = pi.x - q.x, dy = pi.y - q.y, dz = pi.z - q.z;
    const float rr = dot3(dx, dy, dz, dx, dy, dz);
    const float rs = pi.w + q.w;
    if (rr <= h2 && rs > eps && j != k) {
        const float r = sqrtf(rr);
        const float x = fmaf(-r, r, h2);
        const float w = (r >= h) ? 0.0f : c6 * (x * x * x);
        const float coeff = w * __fdividef(two_m, rs);
        sx = fmaf(coeff, vj.x - vi.x, sx);
        sy = fmaf(coeff, vj.y - vi.y, sy);
        sz = fmaf(coeff, vj.z - vi.z, sz);
    }
}

// ---------------------------------------------------------------------------
// XSPH velocity smoothing (correctVelocityXSPH, fluidphysics.cu:355-409):
// post-integration positions, this substep's cell lists and densities.  The
// reference updates velocities in place while neighbours read them (a race);
// here reads see V2 and the result goes to V0 (Jacobi).
// ---------------------------------------------------------------------------
// WALK selects the candidate walk: 0 one loop flattened across the rows, 1 one
// loop per (y,z) row; both visit the same candidates in the same order.  (The
// row-table walk of the force pass measured slower here, 72 registers against
// 54: the pair term is too light to pay for the table.)
// (no __launch_bounds__: with it ptxas caps this kernel at 48 registers and spills)
template <int WALK>
__global__ void k_xsph(const DevParams* __restrict__ params,
                                                   const DevScene* __restrict__ scenes,
                                                   const uint4* __restrict__ tiles,
                                                   const uint32_t* __restrict__ start,
                                                   const float4* __restrict__ P1,
                                                   const float4* __restrict__ P0,
                                                   const float4* __restrict__ V2,
                                                   const uint32_t* __restrict__ mask, size_t mask_stride,
                                                   const uint32_t* __restrict__ maxdisp, float4* __restrict__ V0,
                                                   uint32_t* __restrict__ pend, uint32_t ntiles,
                                                   uint32_t* __restrict__ tile_ctr,
                                                   const uint32_t* __restrict__ status) {
  if (step_failed(status)) return;
  for_each_tile(tiles, ntiles, tile_ctr, [&](const uint4 t) {
    if (threadIdx.x >= t.z) return;
    const uint32_t k = t.y + threadIdx.x;
    const DevScene sc = scenes[t.x];
    const DevParams& pp = params[t.x];
    if (pp.flags & SPH_FLAG_DEFER_XSPH) return;   // the next density pass applies it
    if (threadIdx.x == 0) pend[t.x] = 0u;         // the update is applied here
    const float4 vi = V2[k];
    const float4 old = P1[k];   // the cell this particle was sorted into
    const int3 g = grid_of(pp, old.x, old.y, old.z);
    if (!grid_inside(pp, g)) {
        V0[k] = vi;
        return;
    }
    const float4 pi = P0[k];    // post-integration position, w = density
    const uint32_t delta = sc.part_base - __ldg(start + sc.cell_base);
    const float h2 = pp.h2, h = pp.h, c6 = pp.poly6, two_m = pp.two_mass, eps = pp.eps;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    // The masks hold every candidate within (1 + skin) h at the old
    // positions; a pair can close to h after the move only if the particles
    // moved less than skin*h/2 each, which the force pass recorded.
    uint32_t j;
    const bool masked = __uint_as_float(__ldg(maxdisp)) <= pp.xsph_disp_limit2;
    if (WALK == 1) {
        auto visit = [&](uint32_t jj) { xsph_pair(P0, V2, jj, k, pi, vi, h2, h, c6, two_m, eps, sx, sy, sz); };
        if (masked) for_masked(pp, start, sc.cell_base, delta, g, mask, mask_stride, k, visit);   // skin words 0-8
        else for_candidates(pp, start, sc.cell_base, delta, g, visit);
    } else if (masked) {
        MaskWalk walk(pp, start, sc.cell_base, delta, g, mask, mask_stride, k);   // skin mask, words 0-8
        while (walk.next(j)) xsph_pair(P0, V2, j, k, pi, vi, h2, h, c6, two_m, eps, sx, sy, sz);
    } else {
        RangeWalk walk(pp, start, sc.cell_base, delta, g);
        while (walk.next(j)) xsph_pair(P0, V2, j, k, pi, vi, h2, h, c6, two_m, eps, sx, sy, sz);
    }
    V0[k] = make_float4(fmaf(pp.xsph, sx, vi.x), fmaf(pp.xsph, sy, vi.y), fmaf(pp.xsph, sz, vi.z), 0.f);
  });
}

// ---------------------------------------------------------------------------
// The velocities of a density pass (Vc, cell order) back in the state order
// of the substep before it (slot perm[f]): the export of a scene whose XSPH
// update was pending (packed xyz into `out`, particle perm[f] - base), and its
// materialisation into the state (V0, clearing the scene's pending flag).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(SPH_TILE) k_unsort_vel(const uint4* __restrict__ tiles,
                                                         const uint32_t* __restrict__ perm,
                                                         const float4* __restrict__ Vc, uint32_t base,
                                                         float* __restrict__ out, float4* __restrict__ V0,
                                                         uint32_t* __restrict__ pend,
                                                         const uint32_t* __restrict__ status,
                                                         uint32_t* __restrict__ gate, uint32_t n) {
    const uint4 t = tiles[blockIdx.x];
    // the status word of a force pass run ahead (launch_unsort_vel): it
    // starts failed, so that pass does nothing, when the prefix reported an error
    if (gate && blockIdx.x == 0 && threadIdx.x == 0) *gate = __ldcg(status) != 0u ? SPH_STATUS_SCAN_TIMEOUT : 0u;
    // a failed prefix leaves perm incomplete (the host reports its error)
    if (step_failed(status)) return;
    if (pend && blockIdx.x == 0 && threadIdx.x == 0) pend[t.x] = 0u;
    if (threadIdx.x >= t.z) return;
    const uint32_t f = t.y + threadIdx.x;
    const uint32_t i = __ldg(perm + f);
    if (i - base >= n) return;   // every slot of the scene, once, after a complete prefix
    const float4 v = Vc[f];
    if (out) {
        const size_t o = 3 * (size_t)(i - base);
        out[o] = v.x;
        out[o + 1] = v.y;
        out[o + 2] = v.z;
    }
    if (V0) V0[i] = v;
}

// ---------------------------------------------------------------------------
// Undo a force pass run ahead of the step that takes it: the state before it
// is what the prefix gathered (P1, A1; V1 holds the post-integration
// velocities of a scene whose XSPH update is pending, with its previous cells
// in the w lane), scattered back to the slots it came from.  The force pass
// writes no array the prefix wrote, so the prefix stays valid.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(SPH_TILE) k_undo_ahead(const uint4* __restrict__ tiles,
                                                         const uint32_t* __restrict__ perm,
                                                         const float4* __restrict__ P1,
                                                         const float4* __restrict__ V1,
                                                         const float4* __restrict__ A1, float4* __restrict__ P0,
                                                         float4* __restrict__ V2, float4* __restrict__ A0,
                                                         uint32_t* __restrict__ okey) {
    const uint4 t = tiles[blockIdx.x];
    if (threadIdx.x >= t.z) return;
    const uint32_t f = t.y + threadIdx.x;
    const uint32_t i = __ldg(perm + f);
    const float4 v = V1[f];
    P0[i] = P1[f];
    V2[i] = make_float4(v.x, v.y, v.z, 0.f);
    A0[i] = A1[f];
    okey[i] = __float_as_uint(v.w);
}

// ---------------------------------------------------------------------------
// Host<->device layout helpers and the lattice generator.
// ---------------------------------------------------------------------------
__global__ void k_unpack_state(const float* __restrict__ pos, const float* __restrict__ vel, uint32_t n,
                               uint32_t base, float4* __restrict__ P0, float4* __restrict__ V0,
                               float4* __restrict__ A0, float4* __restrict__ S) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s = base + i;
    P0[s] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0.f);
    V0[s] = vel ? make_float4(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    A0[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    S[s] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Overwrite positions of slots [base, base+n) keeping the rest of the state
// (createFluidBlock writes m_Points element by element, fluidsystem.cu:119-123).
__global__ void k_set_positions(const float* __restrict__ pos, uint32_t n, uint32_t base, float4* __restrict__ P0) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 old = P0[base + i];
    P0[base + i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], old.w);
}

// Export: positions, density colour (DensityColourOperator, fluidutil.cu:67-80)
// and velocities, packed xyz.
__global__ void k_pack_state(const float4* __restrict__ P0, const float4* __restrict__ V0, uint32_t n,
                             uint32_t base, float inv_rest_density, float* __restrict__ pos,
                             float* __restrict__ colour, float* __restrict__ vel) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = P0[base + i];
    const float4 v = V0[base + i];
    if (pos) { pos[3 * i] = p.x; pos[3 * i + 1] = p.y; pos[3 * i + 2] = p.z; }
    if (vel) { vel[3 * i] = v.x; vel[3 * i + 1] = v.y; vel[3 * i + 2] = v.z; }
    if (colour) {
        const float ratio = p.w * inv_rest_density;
        float r = 1.0f, gg = 0.0f, b = 0.0f;
        if (ratio < 1.0f) { r = 0.0f; gg = ratio; b = 1.0f - ratio; }
        else if (ratio < 2.0f) { r = ratio - 1.0f; gg = 2.0f - ratio; b = 0.0f; }
        colour[3 * i] = r; colour[3 * i + 1] = gg; colour[3 * i + 2] = b;
    }
}

// Lattice block with seeded jitter; site (ix,iy,iz) -> particle
// (ix*ny + iy)*nz + iz.  Coordinate: lo + (i + 0.5)*spacing + (2u-1)*jitter.
__global__ void k_lattice(LatticeSpec spec, uint32_t base, float4* __restrict__ P0, float4* __restrict__ V0,
                          float4* __restrict__ A0, float4* __restrict__ S) {
    const uint32_t n = spec.nx * spec.ny * spec.nz;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t iz = i % spec.nz, iy = (i / spec.nz) % spec.ny, ix = i / (spec.nz * spec.ny);
    const uint32_t idx[3] = {ix, iy, iz};
    float c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float u = uniform01(spec.seed, 3ull * i + a);
        const float j = (2.0f * u - 1.0f) * spec.jitter;
        c[a] = (spec.lo[a] + ((float)idx[a] + 0.5f) * spec.spacing) + j;
    }
    const uint32_t s = base + i;
    P0[s] = make_float4(c[0], c[1], c[2], 0.f);
    V0[s] = make_float4(spec.vel[0], spec.vel[1], spec.vel[2], 0.f);
    A0[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    S[s] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Sorted hash for the debug tap: key of the particle now at each slot, with
// the NULL bucket reported as NULL_HASH (m_Hash after the sort).
__global__ void k_sorted_keys(const DevParams* __restrict__ params, const float4* __restrict__ P1, uint32_t n,
                              uint32_t base, uint32_t* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // the cell of the position gathered into slot i by the last sort: the key
    // it was sorted by (the key array itself may already hold the next
    // substep's keys, written by the force pass)
    const float4 p = P1[base + i];
    const uint32_t k = cell_of(*params, p.x, p.y, p.z);
    out[i] = (k == params->ncells) ? SPH_NULL_HASH : k;
}

// ---------------------------------------------------------------------------
// Tile table of a layout: one block per scene writes that scene's tiles
// (scene, first slot, count) from its slot range, starting at tile_first[s].
// The host computes only the per-scene offsets, so a membership change of
// the served form costs O(scenes) on the host instead of O(tiles).
// ---------------------------------------------------------------------------
__global__ void k_build_tiles(const DevScene* __restrict__ scenes, const uint32_t* __restrict__ tile_first,
                              uint32_t tile, uint4* __restrict__ tiles) {
    const uint32_t s = blockIdx.x;
    const DevScene sc = scenes[s];
    const uint32_t first = tile_first[s];
    const uint32_t cnt = (sc.n + tile - 1u) / tile;
    for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
        const uint32_t f = i * tile;
        tiles[first + i] = make_uint4(s, sc.part_base + f, min(tile, sc.n - f), 0u);
    }
}

// ---------------------------------------------------------------------------
// Launch wrappers.
// ---------------------------------------------------------------------------
cudaError_t launch_build_tiles(const DevScene* scenes, const uint32_t* tile_first, uint32_t nscenes, uint32_t tile,
                               uint4* tiles, cudaStream_t st) {
    if (nscenes == 0) return cudaSuccess;
    k_build_tiles<<<nscenes, 128, 0, st>>>(scenes, tile_first, tile, tiles);
    return cudaGetLastError();
}
cudaError_t launch_hash(const StepArgs& a, cudaStream_t st) {
    k_hash<<<a.ntiles, a.block, 0, st>>>(a.params, a.scenes, a.tiles, a.P0, a.count, a.key, a.slot, a.pend, a.okey,
                                         a.status);
    return cudaGetLastError();
}
static inline uint32_t* ctr(const StepArgs& a, int k) { return a.tile_ctr ? a.tile_ctr + k : nullptr; }

// Kernels with a row table in shared memory need 72 B per thread of it; left
// to itself the driver may give them the largest shared-memory carveout and
// shrink L1, which holds the neighbour gathers.  Ask for the smallest carveout
// that still fits 8 blocks of 128 threads (8 x 9 KB + per-block reserve).
cudaError_t init_kernel_attributes() {
    const int pct = SPH_TABLE_CARVEOUT_PCT;
    const void* fns[] = {
        (const void*)k_force_integrate<true, 3, true>, (const void*)k_force_integrate<true, 4, true>,
        (const void*)k_force_integrate<false, 3, true>, (const void*)k_force_integrate<false, 4, true>,
        (const void*)k_normals<true>,
        (const void*)k_density<0, false>, (const void*)k_density<0, true>,
        (const void*)k_density<1, false>, (const void*)k_density<1, true>,
        (const void*)k_density<1, false, true>};
    for (const void* f : fns) {
        const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// a.scan_sums holds at least nt + 2 64-bit words: the tile counter, then one
// look-back descriptor per tile; they start at zero.  With scan_withhold the
// counter starts at 1 instead: the blocks take tiles 1..nt, no block takes
// tile 0, and every wait that reaches tile 0 runs out after scan_spin_limit
// polls (the test of the timeout path).  Tile nt covers no cell (its first
// cell is past n), so it reads and writes no count or start, and its
// descriptor is word nt + 1.
cudaError_t launch_scan(const StepArgs& a, cudaStream_t st) {
    const uint32_t n = a.scan_cells ? a.scan_cells : a.total_cells;
    if (n == 0) return cudaErrorInvalidValue;
    uint32_t* counts = a.count + a.scan_first;
    uint32_t* starts = a.start + a.scan_first;
    const uint32_t vec_ok = ((reinterpret_cast<uintptr_t>(counts) | reinterpret_cast<uintptr_t>(starts)) & 15u) == 0u;
    const uint32_t nt = (n + SCAN_TILE - 1) / SCAN_TILE;
    unsigned long long* desc = reinterpret_cast<unsigned long long*>(a.scan_sums);
    cudaError_t e = cudaMemsetAsync(desc, 0, (size_t)(nt + 2) * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    if (a.scan_withhold) {
        e = cudaMemsetAsync(desc, 1, 1, st);   // the counter's low byte: the next tile handed out is 1
        if (e != cudaSuccess) return e;
    }
    const uint32_t limit = a.scan_spin_limit ? a.scan_spin_limit : SCAN_SPIN_LIMIT;
    k_scan_single<<<nt, SCAN_THREADS, 0, st>>>(counts, n, desc, starts, a.status, a.scan_zeroes_counts, limit,
                                                 vec_ok);
    return cudaGetLastError();
}
cudaError_t launch_scan_raw(const uint32_t* counts, uint32_t n, uint32_t* tile_sums, uint32_t* starts,
                            cudaStream_t st) {
    const uint32_t nt = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (n == 0 || nt > kScanRawMaxTiles) return cudaErrorInvalidValue;
    k_scan_reduce<<<nt, SCAN_THREADS, 0, st>>>(counts, n, tile_sums);
    k_scan_top<<<1, 1024, 0, st>>>(tile_sums, nt);
    k_scan_down<<<nt, SCAN_THREADS, 0, st>>>(counts, n, tile_sums, starts);
    return cudaGetLastError();
}
cudaError_t launch_sort(const StepArgs& a, cudaStream_t st) {
    k_scatter<<<a.ntiles, a.block, 0, st>>>(a.scenes, a.tiles, a.start, a.key, a.slot, a.tmp, a.status);
    k_rank_gather<<<a.ntiles, a.block, 0, st>>>(a.scenes, a.tiles, a.start, a.key, a.tmp, a.P0, a.V0, a.A0, a.V2,
                                                a.okey, a.pend, a.P1, a.V1, a.A1, a.perm, a.status);
    return cudaGetLastError();
}
bool density_split(const StepArgs& a) {
    return (a.variant & SPH_VARIANT_DENSITY_SPLIT) != 0u && (a.variant & SPH_VARIANT_DENSITY_ROWS) != 0u &&
           !a.skin_masks && a.tile_ctr == nullptr && a.particles <= SPH_DENSITY_SPLIT_MAX;
}
cudaError_t launch_density(const StepArgs& a, cudaStream_t st) {
    const size_t smem = (size_t)SPH_ROW_TABLE_WORDS * a.block * sizeof(uint32_t);   // the row table
    if (density_split(a)) {
        k_density<1, false, true><<<a.ntiles, 3u * a.block, smem, st>>>(
            a.params, a.scenes, a.tiles, a.start, a.P1, a.S, a.mask, a.mask_stride, a.V1, a.pend, a.Vc, a.dbg_nbr,
            a.ntiles, nullptr, a.status);
        return cudaGetLastError();
    }
    const bool rows = (a.variant & SPH_VARIANT_DENSITY_ROWS) != 0u;
    auto kern = a.skin_masks ? (rows ? k_density<1, true> : k_density<0, true>)
                             : (rows ? k_density<1, false> : k_density<0, false>);
    kern<<<a.grid_nbr, a.block, smem, st>>>(a.params, a.scenes, a.tiles, a.start, a.P1, a.S, a.mask, a.mask_stride,
                                            a.V1, a.pend, a.Vc, a.dbg_nbr, a.ntiles, ctr(a, 0), a.status);
    return cudaGetLastError();
}
cudaError_t launch_unsort_vel(const StepArgs& a, uint32_t first_tile, uint32_t ntiles, uint32_t base, uint32_t n,
                              float* out, float4* V0, bool clear_pending, cudaStream_t st, uint32_t* gate) {
    if (ntiles == 0) return cudaSuccess;
    k_unsort_vel<<<ntiles, a.block, 0, st>>>(a.tiles + first_tile, a.perm, a.Vc, base, out, V0,
                                             clear_pending ? a.pend : nullptr, a.status, gate, n);
    return cudaGetLastError();
}
cudaError_t launch_undo_ahead(const StepArgs& a, uint32_t first_tile, uint32_t ntiles, cudaStream_t st) {
    if (ntiles == 0) return cudaSuccess;
    k_undo_ahead<<<ntiles, a.block, 0, st>>>(a.tiles + first_tile, a.perm, a.P1, a.V1, a.A1, a.P0, a.V2, a.A0,
                                             a.okey);
    return cudaGetLastError();
}
cudaError_t launch_normals(const StepArgs& a, cudaStream_t st) {
    const bool table = (a.variant & SPH_VARIANT_NORMALS_TABLE) != 0u;
    auto kern = table ? k_normals<true> : k_normals<false>;
    const size_t smem = table ? (size_t)SPH_ROW_TABLE_WORDS * a.block * sizeof(uint32_t) : 0;
    kern<<<a.grid_nbr, a.block, smem, st>>>(a.params, a.scenes, a.tiles, a.start, a.P1, a.S, a.mask, a.mask_stride,
                                            a.N, a.ntiles, ctr(a, 1), a.status);
    return cudaGetLastError();
}
cudaError_t launch_force(const StepArgs& a, cudaStream_t st) {
    const bool occ = (a.variant & SPH_VARIANT_FORCE_OCC) != 0u;
    const bool table = (a.variant & SPH_VARIANT_FORCE_TABLE) != 0u;
    auto kern = a.any_tension
                    ? (table ? (occ ? k_force_integrate<true, 4, true> : k_force_integrate<true, 3, true>)
                             : (occ ? k_force_integrate<true, 4, false> : k_force_integrate<true, 3, false>))
                    : (table ? (occ ? k_force_integrate<false, 4, true> : k_force_integrate<false, 3, true>)
                             : (occ ? k_force_integrate<false, 4, false> : k_force_integrate<false, 3, false>));
    const size_t smem = table ? (size_t)SPH_ROW_TABLE_WORDS * a.block * sizeof(uint32_t) : 0;
    kern<<<a.grid_nbr, a.block, smem, st>>>(a.params, a.scenes, a.tiles, a.start, a.P1, a.Vc, a.A1, a.S, a.N, a.mask,
                                            a.mask_stride, a.P0, a.V2, a.A0, a.skin_masks ? a.maxdisp : nullptr,
                                            a.okey, a.pend, a.count, a.key, a.slot, a.status, a.dbg_forces,
                                            a.ntiles, ctr(a, 2));
    return cudaGetLastError();
}
cudaError_t launch_xsph(const StepArgs& a, cudaStream_t st) {
    auto kern = (a.variant & SPH_VARIANT_XSPH_ROWS) ? k_xsph<1> : k_xsph<0>;
    kern<<<a.grid_nbr, a.block, 0, st>>>(a.params, a.scenes, a.tiles, a.start, a.P1, a.P0, a.V2, a.mask,
                                         a.mask_stride, a.maxdisp, a.V0, a.pend, a.ntiles, ctr(a, 3), a.status);
    return cudaGetLastError();
}
cudaError_t launch_unpack(const float* pos, const float* vel, uint32_t n, uint32_t base, float4* P0, float4* V0,
                          float4* A0, float4* S, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_unpack_state<<<(n + 255) / 256, 256, 0, st>>>(pos, vel, n, base, P0, V0, A0, S);
    return cudaGetLastError();
}
cudaError_t launch_set_positions(const float* pos, uint32_t n, uint32_t base, float4* P0, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_set_positions<<<(n + 255) / 256, 256, 0, st>>>(pos, n, base, P0);
    return cudaGetLastError();
}
cudaError_t launch_pack(const float4* P0, const float4* V0, uint32_t n, uint32_t base, float inv_rest_density,
                        float* pos, float* colour, float* vel, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_pack_state<<<(n + 255) / 256, 256, 0, st>>>(P0, V0, n, base, inv_rest_density, pos, colour, vel);
    return cudaGetLastError();
}
cudaError_t launch_lattice(const LatticeSpec& spec, uint32_t base, float4* P0, float4* V0, float4* A0, float4* S,
                           cudaStream_t st) {
    const uint32_t n = spec.nx * spec.ny * spec.nz;
    if (n == 0) return cudaSuccess;
    k_lattice<<<(n + 255) / 256, 256, 0, st>>>(spec, base, P0, V0, A0, S);
    return cudaGetLastError();
}
cudaError_t launch_sorted_keys(const DevParams* params, const float4* P1, uint32_t n, uint32_t base,
                               uint32_t* out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_sorted_keys<<<(n + 255) / 256, 256, 0, st>>>(params, P1, n, base, out);
    return cudaGetLastError();
}

}  // namespace sph
