// Launch interface of the substep kernels (sph_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "sph_types.h"

namespace sph {

// Device pointers and sizes for one substep over all live scenes.
struct StepArgs {
    const DevParams* params;   // one per scene (indexed by scene table position)
    const DevScene* scenes;
    const uint4* tiles;        // (scene, first slot, count, 0)
    uint32_t ntiles;
    uint32_t particles;        // particles the tiles hold
    uint32_t total_cells;      // packed cell arena size including NULL buckets
    float4 *P0, *V0, *A0;      // state
    float4 *P1, *V1, *A1;      // cell-ordered state
    float4 *V2;                // post-integration velocity (before XSPH)
    float4 *Vc;                // cell-ordered velocities with any pending XSPH update applied
    uint32_t *okey;            // each slot's cell in the last substep (packed; gathered into V1.w)
    uint32_t *pend;            // per scene: its last XSPH update is pending
    float4 *S;                 // (rho, p, c^2, 0)
    float4 *N;                 // normals
    uint32_t *count, *start, *scan_sums;
    uint32_t scan_first;           // the scan covers cells [scan_first, scan_first + scan_cells) (one scene's
    uint32_t scan_cells;           // range for a single scene's prefix; else 0 and total_cells)
    uint32_t scan_zeroes_counts;   // nonzero: the scan leaves every count it read at zero for the next hash
    uint32_t scan_spin_limit;      // polls of one look-back wait before it gives up (SPH_STATUS_SCAN_TIMEOUT)
    uint32_t scan_withhold;        // test control: tile 0 is never handed out, so waits on it run out
    uint32_t *key, *slot, *tmp, *perm;
    uint32_t *status;
    uint32_t *mask;            // SPH_MASK_ROWS neighbour-mask words per slot, word m at mask[m*mask_stride + slot]:
                               // SPH_MASK_SKIN skin radius (XSPH), SPH_MASK_EXACT exact neighbours (normals, forces)
    size_t mask_stride;
    uint32_t *maxdisp;         // largest (displacement/h)^2 of the substep, float bits
    uint32_t block;            // threads per block = particles per tile
    uint32_t grid_nbr;         // blocks of the neighbour passes (ntiles, or the persistent grid)
    uint32_t *tile_ctr;        // 4 tile counters for persistent neighbour passes, or nullptr
    uint32_t variant;          // SPH_VARIANT_* bits: per-row walks, force register budget
    uint32_t any_tension;      // nonzero when some live scene has surface tension on
    uint32_t skin_masks;       // nonzero when some scene runs a per-substep XSPH pass (needs the skin masks)
    uint32_t *dbg_nbr;         // optional: neighbour counts per sorted slot
    float4 *dbg_forces;        // optional: 4 force vectors per sorted slot
};

// Shared-memory carveout (percent of the SM's maximum) requested for the
// kernels that keep a row table in shared memory: the smallest that holds
// the tables of 8 blocks of 128 threads, so that L1 keeps the rest.
#ifndef SPH_TABLE_CARVEOUT_PCT
#define SPH_TABLE_CARVEOUT_PCT 50
#endif
// One-time per-device kernel attributes (call before the first launch).
cudaError_t init_kernel_attributes();

// The tile table of a layout from the scene table: scene s's tiles start at
// tile_first[s] (tiles must hold every scene's ceil(n / tile) entries).
cudaError_t launch_build_tiles(const DevScene* scenes, const uint32_t* tile_first, uint32_t nscenes, uint32_t tile,
                               uint4* tiles, cudaStream_t st);
cudaError_t launch_hash(const StepArgs& a, cudaStream_t st);
cudaError_t launch_scan(const StepArgs& a, cudaStream_t st);
// Cells per scan tile, and the most tiles launch_scan_raw takes (k_scan_top
// scans them in one block of 1024 threads, 32 sums each).
constexpr uint32_t kScanTileCells = 4096u;
constexpr uint32_t kScanRawMaxTiles = 1024u * 32u;
// Exclusive scan of counts[0,n) into starts[0,n] with caller-provided tile
// sums (ceil(n/kScanTileCells) entries, at most kScanRawMaxTiles).
cudaError_t launch_scan_raw(const uint32_t* counts, uint32_t n, uint32_t* tile_sums, uint32_t* starts,
                            cudaStream_t st);
cudaError_t launch_sort(const StepArgs& a, cudaStream_t st);
cudaError_t launch_density(const StepArgs& a, cudaStream_t st);
// Whether launch_density splits the candidate scan (SPH_VARIANT_DENSITY_SPLIT:
// the per-row scan without skin words, one block per tile, and at most
// SPH_DENSITY_SPLIT_MAX particles in the launch).
bool density_split(const StepArgs& a);
cudaError_t launch_normals(const StepArgs& a, cudaStream_t st);
cudaError_t launch_force(const StepArgs& a, cudaStream_t st);
cudaError_t launch_xsph(const StepArgs& a, cudaStream_t st);
// Vc (cell order, over tiles [first_tile, first_tile + ntiles) of one scene
// of n particles) back into state order: packed xyz into `out` (particle
// slot - base) and/or into V0; optionally clears the scene's pending flag.
// Does nothing after a failed prefix.  With `gate`, also
// sets that word up as the status word of a force pass run ahead: failed (the
// pass does nothing) when a.status reports an error.
cudaError_t launch_unsort_vel(const StepArgs& a, uint32_t first_tile, uint32_t ntiles, uint32_t base, uint32_t n,
                              float* out, float4* V0, bool clear_pending, cudaStream_t st, uint32_t* gate = nullptr);
// Undo a force pass run ahead (one scene whose XSPH update was pending, over
// its tiles): P0, V2, A0 and okey back from the prefix's gathered copies.
cudaError_t launch_undo_ahead(const StepArgs& a, uint32_t first_tile, uint32_t ntiles, cudaStream_t st);

cudaError_t launch_unpack(const float* pos, const float* vel, uint32_t n, uint32_t base, float4* P0, float4* V0,
                          float4* A0, float4* S, cudaStream_t st);
cudaError_t launch_set_positions(const float* pos, uint32_t n, uint32_t base, float4* P0, cudaStream_t st);
cudaError_t launch_pack(const float4* P0, const float4* V0, uint32_t n, uint32_t base, float inv_rest_density,
                        float* pos, float* colour, float* vel, cudaStream_t st);
cudaError_t launch_lattice(const LatticeSpec& spec, uint32_t base, float4* P0, float4* V0, float4* A0, float4* S,
                           cudaStream_t st);
cudaError_t launch_sorted_keys(const DevParams* params, const float4* P1, uint32_t n, uint32_t base,
                               uint32_t* out, cudaStream_t st);

}  // namespace sph
