// Allocation-free cell-start scan.
//
// Some callers of this library cannot call cudaMalloc: a host application
// that carves all device memory into its own arena at start-up and forbids
// later allocations, or a real-time frame loop where an allocation or free
// would stall the device.  For them sph_scan_cells_noalloc() turns per-cell
// particle counts into cell starts (the exclusive_scan of
// fluidsystem.cu:316) with every byte of scratch in a fixed array that lives
// in this file, so the call allocates nothing.
//
// The scratch is a file-scope __device__ array of SPH_NOALLOC_MAX_TILES
// tile sums (128 KiB).  Every GPU that loads the library holds it until the
// process exits.  All calls share it and it keeps the last call's contents;
// each call overwrites every tile sum it reads, so nothing needs clearing,
// but calls that overlap on the GPU (different streams or threads) race on
// it and must be serialised by the caller.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sph_c.h"
#include "sph_kernels.h"

static_assert(SPH_NOALLOC_MAX_TILES == sph::kScanRawMaxTiles, "scratch holds every tile sum the scan takes");
static_assert(SPH_NOALLOC_MAX_CELLS == SPH_NOALLOC_MAX_TILES * sph::kScanTileCells, "cell limit");

namespace {

static __device__ __align__(256) uint32_t g_tile_sums[SPH_NOALLOC_MAX_TILES];

// Device address of g_tile_sums in the current device's current context.  In
// host code the name g_tile_sums is only a host-side stand-in, never a device
// address.  It is looked up on every call rather than cached: an application
// that calls cudaDeviceReset gets a new context, and with it a new address,
// so a cached one could point into freed memory.  The lookup is a host-side
// table read once the module is loaded; the first call on a device may load
// the module (lazy loading), which is why that call should come before any
// stream capture.
int scratch_for_current_device(uint32_t** out) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_tile_sums) != cudaSuccess || !p) return SPH_ECUDA;
    *out = static_cast<uint32_t*>(p);
    return SPH_OK;
}

}  // namespace

extern "C" int sph_scan_cells_noalloc(const uint32_t* counts, uint32_t n, uint32_t* starts, void* stream) {
    if (!counts || !starts || n == 0) return SPH_EINVAL;
    if (n > SPH_NOALLOC_MAX_CELLS) return SPH_EINVAL;   // beyond the fixed scratch
    uint32_t* sums = nullptr;
    const int rc = scratch_for_current_device(&sums);
    if (rc != SPH_OK) return rc;
    const cudaError_t e = sph::launch_scan_raw(counts, n, sums, starts, (cudaStream_t)stream);
    return e == cudaSuccess ? SPH_OK : SPH_ECUDA;
}
