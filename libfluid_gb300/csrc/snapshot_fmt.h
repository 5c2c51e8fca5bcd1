// Snapshot byte layout shared by the single-system and batched C ABI:
// a 128-byte sph_snapshot_header, then n float4 positions, n float4
// velocities and n float4 accelerations (the engine's slot arrays verbatim).
#pragma once
#include <cstring>
#include <string>

#include "../../include/sph_c.h"

namespace sph {

static_assert(sizeof(sph_params) == 88, "sph_params layout");
static_assert(sizeof(sph_snapshot_header) == 128, "snapshot header is 128 bytes");

inline uint64_t snapshot_total_bytes(uint32_t n) { return sizeof(sph_snapshot_header) + 48ull * n; }

inline void snapshot_make_header(sph_snapshot_header& h, uint32_t n, const sph_params& p) {
    std::memset(&h, 0, sizeof(h));
    h.magic = SPH_SNAPSHOT_MAGIC;
    h.version = SPH_SNAPSHOT_VERSION;
    h.n = n;
    h.header_bytes = (uint32_t)sizeof(sph_snapshot_header);
    h.params = p;
}

// Validate a snapshot buffer; on success copies its header to *out.
inline bool snapshot_parse(const void* buf, uint64_t bytes, sph_snapshot_header* out, std::string* why) {
    if (!buf || bytes < sizeof(sph_snapshot_header)) { *why = "snapshot shorter than its header"; return false; }
    std::memcpy(out, buf, sizeof(*out));
    if (out->magic != SPH_SNAPSHOT_MAGIC) { *why = "not a snapshot (bad magic)"; return false; }
    if (out->version != SPH_SNAPSHOT_VERSION) { *why = "unsupported snapshot version"; return false; }
    if (out->header_bytes != sizeof(sph_snapshot_header)) { *why = "bad snapshot header size"; return false; }
    if (bytes < snapshot_total_bytes(out->n)) { *why = "snapshot truncated"; return false; }
    return true;
}

}  // namespace sph
