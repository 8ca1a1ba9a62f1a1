// Test harness (host only): runs spk::plan_batch (sparkle_gb300/csrc/batch_plan.h) and checks the invariants
// spk_render_batch relies on. Returns 0 when all hold, else an error code; writes the group count.
#include <cstdint>
#include <vector>

#include "../../sparkle_gb300/csrc/batch_plan.h"

extern "C" int batch_plan_check(const uint64_t *items, const uint32_t *spp, uint32_t n, uint64_t slots, uint32_t min1,
                                uint32_t min2, uint32_t *out_groups) {
    std::vector<uint32_t> queue_base(n, 0xFFFFFFFFu);
    const std::vector<spk::BatchPlanGroup> groups = spk::plan_batch(items, spp, n, slots, min1, min2, queue_base.data());
    *out_groups = static_cast<uint32_t>(groups.size());
    if (n == 0) return groups.empty() ? 0 : 1;
    std::vector<uint64_t> base(n + 1, 0);
    for (uint32_t r = 0; r < n; ++r) base[r + 1] = base[r] + items[r];
    // groups tile the requests and the items in order, each whole requests
    uint32_t next_req = 0;
    for (const spk::BatchPlanGroup &g : groups) {
        if (g.req_lo != next_req || g.req_hi <= g.req_lo || g.req_hi > n) return 2;
        if (g.item_lo != base[g.req_lo] || g.item_hi != base[g.req_hi]) return 3;
        // at most `slots` items, unless the group is one request
        if (g.item_hi - g.item_lo > slots && g.req_hi - g.req_lo != 1) return 4;
        // maximal: the next request would not have fitted
        if (g.req_hi < n && base[g.req_hi + 1] - g.item_lo <= slots) return 5;
        next_req = g.req_hi;
        // first-pass queue: a permutation of 0 .. first-1, each request's items in order from queue_base,
        // requests of spp >= min2 first, then spp >= min1, then the rest
        const uint64_t first = std::min<uint64_t>(slots, g.item_hi - g.item_lo), first_end = g.item_lo + first;
        std::vector<uint8_t> seen(first, 0);
        uint64_t c0 = 0, c01 = 0;
        for (uint32_t r = g.req_lo; r < g.req_hi; ++r) {
            const uint64_t lo = std::min(base[r], first_end), hi = std::min(base[r + 1], first_end);
            for (uint64_t i = lo; i < hi; ++i) {
                const uint64_t q = queue_base[r] + (i - base[r]);
                if (q >= first || seen[q]) return 6;
                seen[q] = 1;
                const int cls = spp[r] >= min2 ? 0 : spp[r] >= min1 ? 1 : 2;
                if ((cls == 0) != (q < g.packet2_items)) return 7;
                if ((cls <= 1) != (q < g.packet_items)) return 8;
            }
            const int cls = spp[r] >= min2 ? 0 : spp[r] >= min1 ? 1 : 2;
            if (cls == 0) c0 += hi - lo;
            if (cls <= 1) c01 += hi - lo;
        }
        for (uint64_t q = 0; q < first; ++q)
            if (!seen[q]) return 9;
        if (c0 != g.packet2_items || c01 != g.packet_items) return 10;
    }
    return next_req == n ? 0 : 11;
}
