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

#include <mutex>

#include "../../include/sph_c.h"
#include "sph_kernels.h"

namespace {

constexpr uint32_t kTile = 4096;                       // cells per scan tile (sph_kernels.cu)
constexpr uint32_t kMaxTiles = SPH_NOALLOC_MAX_TILES;  // one u32 sum per tile

static __device__ __align__(256) uint32_t g_tile_sums[kMaxTiles];

// Device address of g_tile_sums, looked up once per device.  In host code
// the name g_tile_sums is only a host-side stand-in, never a device address.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint32_t* g_addr[kMaxDevices] = {};

int scratch_for_current_device(uint32_t** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SPH_ECUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_tile_sums) != cudaSuccess || !p) return SPH_ECUDA;
        g_addr[dev] = (uint32_t*)p;
    }
    *out = g_addr[dev];
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
