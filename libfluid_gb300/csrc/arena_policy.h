// Sizing policy of the engine's particle and cell arenas (host only, no
// device calls), so that it can be checked on its own.
//
// An engine keeps every live scene in one particle arena and one cell grid.
// Growing either copies (particles) or reallocates (cells) the whole array
// set, so growth is geometric (x1.5), and under a byte budget:
//   - a request whose arrays cannot fit the budget at all is refused
//     (kArenaOverBudget);
//   - when x1.5 would cross the budget, the particle arena grows once to
//     what the budget allows, keeping 1/32 of it for cell growth, instead of
//     to exactly what is asked: a server admitting scene after scene would
//     otherwise copy the whole arena for each of them;
//   - an arena of at least 2^20 slots that could then grow by less than an
//     eighth does not grow (kArenaAtBudget): the caller waits for scenes to
//     leave rather than pay a full copy for a sliver.
#pragma once
#include <stdint.h>

#include <algorithm>

namespace sph {

enum ArenaPlanStatus { kArenaOk = 0, kArenaOverBudget = 1, kArenaAtBudget = 2 };

struct ArenaPlan {
    uint64_t parts;   // particle slots to hold (>= the current capacity)
    uint64_t cells;   // cells to hold (>= the current capacity)
    int status;       // ArenaPlanStatus; on failure parts/cells are the current capacities
};

// parts, cells: what the layout needs; pcap, ccap: current capacities;
// byte_limit: 0 for no budget; bytes_per_particle: device bytes per slot
// (cells cost 8 bytes each).
inline ArenaPlan plan_arena(uint64_t parts, uint64_t cells, uint64_t pcap, uint64_t ccap, uint64_t byte_limit,
                            uint64_t bytes_per_particle) {
    const uint64_t bpp = bytes_per_particle;
    if (byte_limit && std::max(parts, pcap) * bpp + std::max(cells, ccap) * 8 > byte_limit)
        return {pcap, ccap, kArenaOverBudget};
    uint64_t np = pcap;
    if (parts > pcap) {
        np = std::max<uint64_t>(parts, pcap + pcap / 2);
        if (byte_limit && np * bpp + std::max(cells, ccap) * 8 > byte_limit) {
            const uint64_t cell_bytes = std::max(cells, ccap) * 8 + byte_limit / 32;
            const uint64_t room = byte_limit > cell_bytes ? (byte_limit - cell_bytes) / bpp : 0;
            np = std::max(parts, std::min(np, room));
            if (pcap >= (1u << 20) && np < pcap + pcap / 8) return {pcap, ccap, kArenaAtBudget};
        }
    }
    uint64_t nc = ccap;
    if (cells > ccap) {
        nc = std::max<uint64_t>(cells, ccap + ccap / 2);
        if (byte_limit && np * bpp + nc * 8 > byte_limit) {
            const uint64_t used = np * bpp;
            nc = std::max(cells, std::min(nc, byte_limit > used ? (byte_limit - used) / 8 : 0));
        }
    }
    return {np, nc, kArenaOk};
}

}  // namespace sph
